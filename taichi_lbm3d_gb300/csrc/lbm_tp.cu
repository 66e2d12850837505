// K4: two-phase colour-gradient step (2phase/lbm_solver_3d_2phase_sparse.py, "TP").
//
// The reference's step (TP:626-632) is colission (MRT + colour gradient + CapA
// surface tension + recolouring + colour push, :302-373), streaming1,
// Boundary_condition, streaming3 (macros, colour sums, psi, :587-606) and
// Boundary_condition_psi (:445-487).  Collision at a node needs psi at its
// neighbours *after* the previous step, so one step is two launches:
//
//   A  tp_colour_kernel: pull the colour distributions.  rho_r(y) = sum over s
//      of g_r(y - e_s)[s] (or g_r(y)[LR[s]] when y - e_s is solid), g recomputed
//      at the source from its stored (rho_r, rho_b, v) and its 9 recolouring
//      amounts; then psi = rho_r - rho_b/(rho_r + rho_b) (TP:606, kept as the
//      reference writes it) and constant-psi faces.
//   B  tp_flow_kernel: gather F, face BCs, macros; colour gradient C from psi of
//      the neighbours (clamped on constant-psi faces, TP:390-429); psi-dependent
//      relaxation (TP:278-300); CapA terms in meq (TP:316-322); MRT + script Guo;
//      store f, v, rho and the node's 9 recolouring amounts (TP:352-364) for the
//      next step's launch A.
//
// The colour sums are taken in direction order 0..18, one of the orders the
// reference's atomic += can produce; the CPU oracle uses the same order, so
// the two agree bit for bit.  Per node and step the launches move the 152 B of
// FP32 populations plus rho_r, rho_b, psi, v and the recolouring amounts.
#include <cuda_runtime.h>

#include <vector>

#include "lbm_kernels.cuh"

namespace {
using namespace lbmk;

template <typename R>
struct TpConsts {
    SpConsts<R> sp;
    R wl, wg, lg0, l1, l2, g1, g2;  // TP:102-110, folded to R
    R psi_solid, capa, hcapa;       // hcapa = 0.5 * capa
    int32_t psi_bc[6];
    int32_t any_psi_bc;
    R psi_val[6], psi_rr[6], psi_rb[6];
};

// Compute_S_local (TP:278-300): s_v and s_other from psi.
template <typename R>
__device__ __forceinline__ void s_local(const TpConsts<R>& T, R psi, R& sv, R& so) {
    if (psi > (R)0) {
        if (psi > (R)0.1) sv = T.wl;
        else sv = (T.lg0 + T.l1 * psi) + (T.l2 * psi) * psi;
    } else {
        if (psi < (R)-0.1) sv = T.wg;
        else sv = (T.lg0 + T.g1 * psi) + (T.g2 * psi) * psi;
    }
    so = ((R)8.0 * ((R)2.0 - sv)) / ((R)8.0 - sv);
}

// periodic_index_for_psi (TP:390-429) for one coordinate.
__device__ __forceinline__ int psi_wrap(int x, int n, int bc_lo, int bc_hi) {
    if (x < 0) return bc_lo == 0 ? n - 1 : 0;
    if (x > n - 1) return bc_hi == 0 ? 0 : n - 1;
    return x;
}

// Compute_C (TP:259-276): C = sum_s 3 w_s e_s psi(x + e_s), psi_solid at solid
// neighbours; zero when |rho_r - rho_b| > 0.9 next to a solid.
template <typename R>
__device__ __forceinline__ void colour_gradient(const TpConsts<R>& T, const int32_t* __restrict__ map,
                                                const R* __restrict__ psi, int i, int j, int k, R rr, R rb, R& Cx,
                                                R& Cy, R& Cz) {
    const int nx = T.sp.nx, ny = T.sp.ny, nz = T.sp.nz;
    const int xm = psi_wrap(i - 1, nx, T.psi_bc[0], T.psi_bc[1]), xp = psi_wrap(i + 1, nx, T.psi_bc[0], T.psi_bc[1]);
    const int ym = psi_wrap(j - 1, ny, T.psi_bc[2], T.psi_bc[3]), yp = psi_wrap(j + 1, ny, T.psi_bc[2], T.psi_bc[3]);
    const int zm = psi_wrap(k - 1, nz, T.psi_bc[4], T.psi_bc[5]), zp = psi_wrap(k + 1, nz, T.psi_bc[4], T.psi_bc[5]);
    Cx = (R)0;
    Cy = (R)0;
    Cz = (R)0;
    bool touch = false;
#pragma unroll
    for (int s = 1; s < 19; ++s) {
        const int ex = lbm_ex(s), ey = lbm_ey(s), ez = lbm_ez(s);
        const int x = ex > 0 ? xp : (ex < 0 ? xm : i);
        const int y = ey > 0 ? yp : (ey < 0 ? ym : j);
        const int z = ez > 0 ? zp : (ez < 0 ? zm : k);
        const int nb = __ldg(map + x + nx * (y + ny * z));
        R ps;
        if (nb >= 0) {
            ps = psi[nb];
        } else {
            ps = T.psi_solid;
            touch = true;
        }
        const R t = ((R)3.0 * (R)lbm_w(s)) * ps;
        if (ex != 0) Cx = ex > 0 ? Cx + t : Cx - t;
        if (ey != 0) Cy = ey > 0 ? Cy + t : Cy - t;
        if (ez != 0) Cz = ez > 0 ? Cz + t : Cz - t;
    }
    R dr = rr - rb;
    if (dr < (R)0) dr = -dr;
    if (dr > (R)0.9 && touch) {
        Cx = (R)0;
        Cy = (R)0;
        Cz = (R)0;
    }
}

// Recolouring amounts of the 9 opposite pairs (TP:346-364): cospsi_p for
// kk = 2p+1; zero when |C| = 0 (no recolouring).
template <typename R>
__device__ __forceinline__ void recolour_amounts(R rr, R rb, R vx, R vy, R vz, R Cx, R Cy, R Cz, R cc, R* cs) {
    const R uv = lbm_usq(vx, vy, vz);
#define LBM_RC(P)                                                                           \
    {                                                                                       \
        constexpr int kk = 2 * P + 1;                                                       \
        R cp = (R)0;                                                                        \
        if (cc > (R)0) {                                                                    \
            const R ga = lbm_feq<kk, R>(rr, vx, vy, vz, uv), gb = lbm_feq<kk + 1, R>(rr, vx, vy, vz, uv); \
            const R ba = lbm_feq<kk, R>(rb, vx, vy, vz, uv), bb = lbm_feq<kk + 1, R>(rb, vx, vy, vz, uv); \
            const R ef = lbm_edot<kk, R>(Cx, Cy, Cz);                                       \
            cp = ga < gb ? ga : gb;                                                         \
            cp = cp < ba ? cp : ba;                                                         \
            cp = cp < bb ? cp : bb;                                                         \
            cp = cp * (ef / cc);                                                            \
        }                                                                                   \
        cs[P] = cp;                                                                         \
    }
    LBM_RC(0) LBM_RC(1) LBM_RC(2) LBM_RC(3) LBM_RC(4) LBM_RC(5) LBM_RC(6) LBM_RC(7) LBM_RC(8)
#undef LBM_RC
}

// Two-phase MRT collision (TP:302-344) of F in place.
template <typename R, bool FORCE, bool FAST>
__device__ __forceinline__ void collide_tp(R* F, R r, R vx, R vy, R vz, R cc, R n0, R n1, R n2, R sv, R so,
                                           const TpConsts<R>& T) {
    R m[19];
    if constexpr (FAST) mrt_moments_fast<R>(F, m);
    else mrt_moments<R>(F, m);
    R meq[19];
#pragma unroll
    for (int s = 0; s < 19; ++s) meq[s] = (R)0;
    meq[0] = r; meq[3] = vx; meq[5] = vy; meq[7] = vz;
    meq[1] = lbm_usq(vx, vy, vz);
    meq[9] = (((R)2 * vx) * vx - vy * vy) - vz * vz;
    meq[11] = vy * vy - vz * vz;
    meq[13] = vx * vy; meq[14] = vy * vz; meq[15] = vx * vz;
    const R hc = T.hcapa * cc;
    meq[1] = meq[1] + T.capa * cc;
    meq[9] = meq[9] + hc * ((((R)2 * n0) * n0 - n1 * n1) - n2 * n2);
    meq[11] = meq[11] + hc * (n1 * n1 - n2 * n2);
    meq[13] = meq[13] + hc * (n0 * n1);
    meq[14] = meq[14] + hc * (n1 * n2);
    meq[15] = meq[15] + hc * (n0 * n2);
#pragma unroll
    for (int s = 0; s < 19; ++s) {
        const int kd = lbm_skind(s);
        if (kd == 0) continue;
        const R S = kd == 1 ? sv : so;
        if constexpr (FAST) m[s] = lbm_fma<R>(S, meq[s] - m[s], m[s]);
        else m[s] = m[s] - S * (m[s] - meq[s]);
    }
    if constexpr (FORCE) {
        const R fx = T.sp.fext[0], fy = T.sp.fext[1], fz = T.sp.fext[2];
        R G[19];
#pragma unroll
        for (int l = 0; l < 19; ++l) {
            R a = ((R)lbm_ex(l) - vx) * fx;
            a = a + ((R)lbm_ey(l) - vy) * fy;
            a = a + ((R)lbm_ez(l) - vz) * fz;
            R eu, ef;
            switch (l) {
#define LBM_EU(S) case S: eu = lbm_edot<S, R>(vx, vy, vz); ef = lbm_edot<S, R>(fx, fy, fz); break;
                LBM_EU(0) LBM_EU(1) LBM_EU(2) LBM_EU(3) LBM_EU(4) LBM_EU(5) LBM_EU(6) LBM_EU(7) LBM_EU(8) LBM_EU(9)
                LBM_EU(10) LBM_EU(11) LBM_EU(12) LBM_EU(13) LBM_EU(14) LBM_EU(15) LBM_EU(16) LBM_EU(17) LBM_EU(18)
#undef LBM_EU
            }
            G[l] = (R)lbm_w(l) * (a + eu * ef);  // GuoF, TP:242-248
        }
        R fg[19];
        if constexpr (FAST) mrt_moments_fast<R>(G, fg);
        else mrt_moments<R>(G, fg);
#pragma unroll
        for (int s = 0; s < 19; ++s) {
            const int kd = lbm_skind(s);
            const R S = kd == 0 ? (R)0 : (kd == 1 ? sv : so);
            if constexpr (FAST) m[s] = lbm_fma<R>((R)1 - (R)0.5 * S, fg[s], m[s]);
            else m[s] = m[s] + ((R)1 - (R)0.5 * S) * fg[s];
        }
    }
    if constexpr (FAST) mrt_back_fast<R>(m, F);
    else mrt_back<R>(m, F);
}

// Everything B does after the macros: colour gradient, collision, recolouring.
template <int STORE, bool FORCE>
__device__ __forceinline__ void tp_collide_and_store(typename Codec<STORE>::R* F, typename Codec<STORE>::R r,
                                                     typename Codec<STORE>::R vx, typename Codec<STORE>::R vy,
                                                     typename Codec<STORE>::R vz, int n, int i, int j, int k,
                                                     const TpConsts<typename Codec<STORE>::R>& T,
                                                     const int32_t* __restrict__ map,
                                                     const typename Codec<STORE>::R* __restrict__ psi,
                                                     typename Codec<STORE>::R rr, typename Codec<STORE>::R rb,
                                                     typename Codec<STORE>::T* __restrict__ fout,
                                                     typename Codec<STORE>::R* __restrict__ cs_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    R Cx, Cy, Cz;
    colour_gradient<R>(T, map, psi, i, j, k, rr, rb, Cx, Cy, Cz);
    const R cc = sqrt(lbm_usq(Cx, Cy, Cz));
    R n0 = (R)0, n1 = (R)0, n2 = (R)0;
    if (cc > (R)0) {
        n0 = Cx / cc;
        n1 = Cy / cc;
        n2 = Cz / cc;
    }
    R sv, so;
    s_local<R>(T, psi[n], sv, so);
    collide_tp<R, FORCE, Cd::DEV>(F, r, vx, vy, vz, cc, n0, n1, n2, sv, so, T);
    store_node<STORE>(F, fout, n, lbm_ref_at(sp_ref(T.sp), i), T.sp.seed);
    R cs[9];
    recolour_amounts<R>(rr, rb, vx, vy, vz, Cx, Cy, Cz, cc, cs);
    const int64_t np = T.sp.np;
#pragma unroll
    for (int p = 0; p < 9; ++p) cs_out[p * np + n] = cs[p];
}

// Programmatic dependent launch between the step's launches (A, B, next A):
// a launch's CTAs may become resident while the previous launch drains; they
// load their coordinates, then wait for it to complete before touching any
// state (the wait returns at once for a launch without the attribute).
__device__ __forceinline__ void tp_pdl_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void tp_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename K, typename... Args>
cudaError_t tp_launch_pdl(K kernel, int grid, int block, cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---------------------------------------------------------------- launch A
template <int Q, typename R>
__device__ __forceinline__ void colour_pull_one(const TpConsts<R>& T, const int32_t* __restrict__ map,
                                                const Rows& rows, int n, int i, int xm, int xp, bool xwrap,
                                                const R* __restrict__ rr, const R* __restrict__ rb,
                                                const R* __restrict__ v, const R* __restrict__ cs, R& acc_r,
                                                R& acc_b) {
    const int64_t np = T.sp.np;
    int src = n;
    if constexpr (Q != 0) {
        constexpr int ex = lbm_ex(Q), ey = lbm_ey(Q), ez = lbm_ez(Q);
        const int row = rows.r[1 - ey][1 - ez];
        const int x = ex > 0 ? xm : (ex < 0 ? xp : i);
        src = xwrap ? __ldg(map + (row - i + x)) : __ldg(map + row - ex);
    }
    const bool bounce = src < 0;
    const int m = bounce ? n : src;
    const R vx = v[m], vy = v[np + m], vz = v[2 * np + m];
    const R uv = lbm_usq(vx, vy, vz);
    R eu = lbm_edot<Q, R>(vx, vy, vz);
    if (bounce) eu = -eu;  // direction LR[Q] at the node itself: e_LR = -e_Q
    R t = (R)1.0 + (R)3.0 * eu;
    t = t + ((R)4.5 * eu) * eu;
    t = t - (R)1.5 * uv;
    R gr = ((R)lbm_w(Q) * rr[m]) * t;
    R gb = ((R)lbm_w(Q) * rb[m]) * t;
    if constexpr (Q != 0) {
        // pair kk = 2p+1 gets +cospsi for red (kk) and -cospsi (kk+1); blue opposite
        const R c = cs[((Q - 1) >> 1) * np + m];
        const bool plus = ((Q & 1) != 0) != bounce;
        gr = plus ? gr + c : gr - c;
        gb = plus ? gb - c : gb + c;
    }
    acc_r = acc_r + gr;
    acc_b = acc_b + gb;
}

// 4 CTAs of 256 per SM (64 registers): the 19 source gathers of 6 values each
// stay in flight together; at the compiler's own 40 registers (6 CTAs) the
// 131^3 drainage step runs 4.7% slower, at 80 registers (3 CTAs) 23% slower.
template <typename R>
__global__ void __launch_bounds__(256, 4) tp_colour_kernel(const __grid_constant__ TpConsts<R> T,
                                                        const R* __restrict__ rr_in, const R* __restrict__ rb_in,
                                                        const R* __restrict__ v, const R* __restrict__ cs,
                                                        R* __restrict__ rr_out, R* __restrict__ rb_out,
                                                        R* __restrict__ psi_out, const int32_t* __restrict__ map,
                                                        const uint32_t* __restrict__ coord) {
    tp_pdl_launch_dependents();
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= T.sp.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
    const int nx = T.sp.nx, ny = T.sp.ny, nz = T.sp.nz;
    const int xm = i == 0 ? nx - 1 : i - 1, xp = i == nx - 1 ? 0 : i + 1;
    const int ym = j == 0 ? ny - 1 : j - 1, yp = j == ny - 1 ? 0 : j + 1;
    const int zm = k == 0 ? nz - 1 : k - 1, zp = k == nz - 1 ? 0 : k + 1;
    const Rows rows = make_rows(nx, ny, i, j, k, ym, yp, zm, zp);
    const bool xwrap = !(i > 0 && i < nx - 1);
    tp_pdl_wait();  // v, cs of the previous flow launch; psi is rewritten below
    R ar = (R)0, ab = (R)0;
#define LBM_CP(Q) colour_pull_one<Q, R>(T, map, rows, n, i, xm, xp, xwrap, rr_in, rb_in, v, cs, ar, ab);
    LBM_CP(0) LBM_ALL_DIRS(LBM_CP)
#undef LBM_CP
    R psi = ar - ab / (ar + ab);  // TP:606 as written
    if (T.any_psi_bc) {
#pragma unroll 1
        for (int f = 0; f < 6; ++f) {
            if (!T.psi_bc[f]) continue;
            const int hi = f & 1;
            const int c = f < 2 ? i : (f < 4 ? j : k);
            const int nmax = f < 2 ? nx : (f < 4 ? ny : nz);
            if (c != (hi ? nmax - 1 : 0)) continue;
            psi = T.psi_val[f];
            ar = T.psi_rr[f];
            ab = T.psi_rb[f];
        }
    }
    rr_out[n] = ar;
    rb_out[n] = ab;
    psi_out[n] = psi;
}

// ---------------------------------------------------------------- launch B
template <int STORE, bool FORCE>
__global__ void __launch_bounds__(256) tp_flow_kernel(const __grid_constant__ TpConsts<typename Codec<STORE>::R> T,
                                                      const typename Codec<STORE>::T* __restrict__ fin,
                                                      typename Codec<STORE>::T* __restrict__ fout,
                                                      const int32_t* __restrict__ map,
                                                      const uint32_t* __restrict__ coord,
                                                      typename Codec<STORE>::R* __restrict__ v,
                                                      typename Codec<STORE>::R* __restrict__ rho_out,
                                                      const typename Codec<STORE>::R* __restrict__ rr,
                                                      const typename Codec<STORE>::R* __restrict__ rb,
                                                      const typename Codec<STORE>::R* __restrict__ psi,
                                                      typename Codec<STORE>::R* __restrict__ cs_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const SpConsts<R>& C = T.sp;
    tp_pdl_launch_dependents();
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
    const int64_t np = C.np;
    tp_pdl_wait();  // rho_r, rho_b, psi of the colour launch; f, v, cs of the previous step
    R F[19];
    gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k, sp_ref(C));
    if (C.any_bc && on_face(i, j, k, C, false)) apply_faces<R, Cd::DEV>(F, i, j, k, n, C, map, v);  // v: previous step
    R r = F[0];
#pragma unroll
    for (int s = 1; s < 19; ++s) r = r + F[s];
    const R rho = Cd::DEV ? (R)1 + r : r;
    R vx = vsum<0>(F), vy = vsum<1>(F), vz = vsum<2>(F);
    vx = vx / rho;
    vy = vy / rho;
    vz = vz / rho;
    if constexpr (FORCE) {
        vx = vx + C.fhalf[0] / rho;
        vy = vy + C.fhalf[1] / rho;
        vz = vz + C.fhalf[2] / rho;
    }
    rho_out[n] = rho;
    v[n] = vx;
    v[np + n] = vy;
    v[2 * np + n] = vz;
    tp_collide_and_store<STORE, FORCE>(F, r, vx, vy, vz, n, i, j, k, T, map, psi, rr[n], rb[n], fout, cs_out);
}

// Initial state (TP:174-187) and the first collision: rho = 1, v = 0, F = feq(1, 0),
// rho_r = (psi + 1)/2, rho_b = 1 - rho_r, psi = the input psi.
template <int STORE, bool FORCE>
__global__ void tp_init_kernel(const __grid_constant__ TpConsts<typename Codec<STORE>::R> T,
                               typename Codec<STORE>::T* __restrict__ fout, const int32_t* __restrict__ map,
                               const uint32_t* __restrict__ coord, typename Codec<STORE>::R* __restrict__ v,
                               typename Codec<STORE>::R* __restrict__ rho_out, typename Codec<STORE>::R* __restrict__ rr,
                               typename Codec<STORE>::R* __restrict__ rb, const typename Codec<STORE>::R* __restrict__ psi,
                               typename Codec<STORE>::R* __restrict__ cs_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= T.sp.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);
    const int64_t np = T.sp.np;
    const R r0 = (psi[n] + (R)1.0) / (R)2.0;
    const R b0 = (R)1.0 - r0;
    rr[n] = r0;
    rb[n] = b0;
    v[n] = (R)0;
    v[np + n] = (R)0;
    v[2 * np + n] = (R)0;
    rho_out[n] = (R)1.0;
    R F[19];
    if constexpr (Cd::DEV) lbm_feq_dev_all<R>((R)0, (R)0, (R)0, (R)0, F);
    else lbm_feq_all<R>((R)1.0, (R)0, (R)0, (R)0, F);
    tp_collide_and_store<STORE, FORCE>(F, Cd::DEV ? (R)0 : (R)1.0, (R)0, (R)0, (R)0, n, lbm_pi(pc), lbm_pj(pc),
                                       lbm_pk(pc), T, map, psi, r0, b0, fout, cs_out);
}

template <typename R>
TpConsts<R> make_tp(const LbmHandle* h) {
    const LbmParams& p = h->p;
    TpConsts<R> T{};
    T.sp = sp_make_consts<R>(h);
    const double wl = 1.0 / (p.niu_l / (1.0 / 3.0) + 0.5);
    const double wg = 1.0 / (p.niu_g / (1.0 / 3.0) + 0.5);
    const double lg0 = 2 * wl * wg / (wl + wg);
    const double l1 = 2 * (wl - lg0) * 10, l2 = -l1 / 0.2;
    const double g1 = 2 * (lg0 - wg) * 10, g2 = g1 / 0.2;
    T.wl = (R)wl; T.wg = (R)wg; T.lg0 = (R)lg0; T.l1 = (R)l1; T.l2 = (R)l2; T.g1 = (R)g1; T.g2 = (R)g2;
    T.psi_solid = (R)p.psi_solid;
    T.capa = (R)p.cap_a;
    T.hcapa = (R)0.5 * T.capa;
    T.any_psi_bc = 0;
    for (int f = 0; f < 6; ++f) {
        T.psi_bc[f] = p.psi_bc[f];
        T.any_psi_bc |= p.psi_bc[f] != 0;
        T.psi_val[f] = (R)p.psi_val[f];
        T.psi_rr[f] = (T.psi_val[f] + (R)1.0) / (R)2.0;
        T.psi_rb[f] = (R)1.0 - T.psi_rr[f];
    }
    return T;
}

template <int STORE>
int tp_init_t(LbmHandle* h) {
    using R = typename Codec<STORE>::R;
    using Tt = typename Codec<STORE>::T;
    const TpConsts<R> T = make_tp<R>(h);
    // psi of the fluid nodes, in node order
    int rc = geom_host_index(h);
    if (rc) return rc;
    std::vector<R> hp(h->np, (R)0);
    for (int32_t n = 0; n < h->n_fluid; ++n) hp[n] = (R)h->psi0[h->cell_of_node[n]];
    rc = lbm_cuda_check(h, cudaMemcpyAsync(h->d_psi, hp.data(), sizeof(R) * h->np, cudaMemcpyHostToDevice, h->stream),
                            "copy psi");
    if (rc) return rc;
    h->cur = 0;
    h->ccur = 0;
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    auto k = h->force ? tp_init_kernel<STORE, true> : tp_init_kernel<STORE, false>;
    k<<<grid, h->block, 0, h->stream>>>(T, (Tt*)h->d_f[0], h->d_map, h->d_coord, (R*)h->d_v, (R*)h->d_rho,
                                        (R*)h->d_rr[0], (R*)h->d_rb[0], (const R*)h->d_psi, (R*)h->d_cs);
    rc = lbm_cuda_check(h, cudaGetLastError(), "tp_init_kernel launch");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "tp_init");
    return rc;
}

template <int STORE>
int tp_steps_t(LbmHandle* h, int32_t nsteps) {
    using R = typename Codec<STORE>::R;
    using Tt = typename Codec<STORE>::T;
    TpConsts<R> T = make_tp<R>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    auto kb = h->force ? tp_flow_kernel<STORE, true> : tp_flow_kernel<STORE, false>;
    for (int32_t it = 0; it < nsteps; ++it) {
        T.sp.seed = (uint32_t)(h->steps_done + it);   // global step index: rounding bits of this step
        const int c = h->ccur;
        cudaError_t e = tp_launch_pdl(tp_colour_kernel<R>, grid, h->block, h->stream, T, (const R*)h->d_rr[c],
                                      (const R*)h->d_rb[c], (const R*)h->d_v, (const R*)h->d_cs, (R*)h->d_rr[c ^ 1],
                                      (R*)h->d_rb[c ^ 1], (R*)h->d_psi, (const int32_t*)h->d_map,
                                      (const uint32_t*)h->d_coord);
        int rc = lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "tp_colour_kernel launch");
        if (rc) return rc;
        h->ccur ^= 1;
        e = tp_launch_pdl(kb, grid, h->block, h->stream, T, (const Tt*)h->d_f[h->cur], (Tt*)h->d_f[h->cur ^ 1],
                          (const int32_t*)h->d_map, (const uint32_t*)h->d_coord, (R*)h->d_v, (R*)h->d_rho,
                          (const R*)h->d_rr[h->ccur], (const R*)h->d_rb[h->ccur], (const R*)h->d_psi, (R*)h->d_cs);
        rc = lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "tp_flow_kernel launch");
        if (rc) return rc;
        h->cur ^= 1;
    }
    return LBM_OK;
}

}  // namespace

int tp_launch_init(LbmHandle* h) {
    if (h->n_fluid == 0) {   // all solid: nothing to initialise (an empty grid is not launchable)
        h->cur = 0;
        h->ccur = 0;
        return LBM_OK;
    }
    switch (h->p.storage) {
    case LBM_STORE_F32: return tp_init_t<LBM_STORE_F32>(h);
    case LBM_STORE_F16_DEV: return tp_init_t<LBM_STORE_F16_DEV>(h);
    case LBM_STORE_BF16_DEV: return tp_init_t<LBM_STORE_BF16_DEV>(h);
    case LBM_STORE_F32_DEV: return tp_init_t<LBM_STORE_F32_DEV>(h);
    case LBM_STORE_F64: return tp_init_t<LBM_STORE_F64>(h);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}

int tp_launch_steps(LbmHandle* h, int32_t n, bool) {
    if (h->n_fluid == 0) return LBM_OK;
    switch (h->p.storage) {
    case LBM_STORE_F32: return tp_steps_t<LBM_STORE_F32>(h, n);
    case LBM_STORE_F16_DEV: return tp_steps_t<LBM_STORE_F16_DEV>(h, n);
    case LBM_STORE_BF16_DEV: return tp_steps_t<LBM_STORE_BF16_DEV>(h, n);
    case LBM_STORE_F32_DEV: return tp_steps_t<LBM_STORE_F32_DEV>(h, n);
    case LBM_STORE_F64: return tp_steps_t<LBM_STORE_F64>(h, n);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}
