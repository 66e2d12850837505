// K1: fused single-phase D3Q19 MRT step over the compacted fluid-node list.
//
// One thread per fluid node, one launch per time step.  A launch performs, for
// its node, the reference's four sweeps rotated into pull form (state between
// launches = post-collision populations f):
//   gather   F[s] = f(x - e_s)[s], or f(x)[LR[s]] when x - e_s is solid
//            (streaming1 push + halfway bounce-back, SP:259-269, periodic wrap Q6)
//   faces    fixed-pressure / fixed-velocity overwrite in face order (SP:272-370)
//   macros   rho, v (+ F/2 rho) (streaming3, SP:372-392)
//   collide  m = M F; m -= S (m - meq); Guo term; f = M^-1 m (colission, SP:222-241)
// Paths: SP = Single_phase/LBM_3D_SinglePhase_Solver.py (taichi_LBM3D tree).
//
// Memory layout (HBM): populations SoA [19][np] in two buffers (ping-pong),
// np = n_fluid padded to 64; dense int32 map cell -> node (or -1 for solid);
// packed node coordinates.  Per node and step the kernel moves 19 loads + 19
// stores of populations (152 B in FP32, 76 B in 16-bit storage), 4 B of
// coordinates and the neighbour map rows (mostly L1/L2 hits).
#include <cuda_runtime.h>

#include "lbm_common.cuh"
#include "lbm_internal.h"

// Resident CTAs per SM requested for the unforced FP32/16-bit step kernel
// (caps registers at 65536 / (256 * LBM_SP_MINBLOCKS)).
#ifndef LBM_SP_MINBLOCKS
#define LBM_SP_MINBLOCKS 6
#endif

namespace {

// Pull sources.  For node x and direction S the population comes from the
// node at x - e_S (periodic wrap, SP:247-257), or -- when that cell is solid --
// from the node's own LR[S] slot (halfway bounce-back, SP:265-268).  The cell is
// looked up in the dense map through 9 row offsets (one per (y, z) pair); when
// no lane of the warp sits on an x face the x neighbours are at +-1 from the
// row offset, so each lookup is one load with an immediate offset.
struct Rows {
    int r[3][3];  // [source y: j-1, j, j+1 wrapped][source z], cell index of (i, y, z)
};

__device__ __forceinline__ Rows make_rows(int nx, int ny, int i, int j, int k, int ym, int yp, int zm, int zp) {
    Rows R;
    const int ys[3] = {ym, j, yp};
    const int zs[3] = {zm, k, zp};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) R.r[a][b] = i + nx * (ys[a] + ny * zs[b]);
    return R;
}

template <int STORE, bool XWRAP>
struct Gather {
    using Cd = Codec<STORE>;
    using T = typename Cd::T;
    using R = typename Cd::R;
    template <int S>
    static __device__ __forceinline__ void one(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* __restrict__ map, const Rows& rows, int i, int xm,
                                               int xp) {
        constexpr int ex = lbm_ex(S), ey = lbm_ey(S), ez = lbm_ez(S);
        // source is x - e_S: row index 0 holds y-1 (used when ey = +1)
        const int row = rows.r[1 - ey][1 - ez];
        int src;
        if constexpr (XWRAP) {
            const int x = ex > 0 ? xm : (ex < 0 ? xp : i);
            src = __ldg(map + (row - i + x));
        } else {
            src = __ldg(map + row - ex);
        }
        if (src >= 0) F[S] = Cd::template dec<S>(fin[lbm_eoff32(src) + 32 * S]);
        else F[S] = Cd::template dec<S>(own[32 * lbm_lr(S)]);
    }
    static __device__ __forceinline__ void all(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* __restrict__ map, const Rows& rows, int i, int xm,
                                               int xp) {
        F[0] = Cd::template dec<0>(own[0]);
#define LBM_G(S) one<S>(F, fin, own, map, rows, i, xm, xp);
        LBM_G(1) LBM_G(2) LBM_G(3) LBM_G(4) LBM_G(5) LBM_G(6) LBM_G(7) LBM_G(8) LBM_G(9)
        LBM_G(10) LBM_G(11) LBM_G(12) LBM_G(13) LBM_G(14) LBM_G(15) LBM_G(16) LBM_G(17) LBM_G(18)
#undef LBM_G
    }
};

// Gather F for node n; warps with no lane on an x face take the immediate-offset path.
template <int STORE>
__device__ __forceinline__ void gather_node(typename Codec<STORE>::R* F, const typename Codec<STORE>::T* __restrict__ fin,
                                            const int32_t* __restrict__ map, int n, int nx, int ny, int nz, int i, int j,
                                            int k) {
    const int xm = i == 0 ? nx - 1 : i - 1, xp = i == nx - 1 ? 0 : i + 1;
    const int ym = j == 0 ? ny - 1 : j - 1, yp = j == ny - 1 ? 0 : j + 1;
    const int zm = k == 0 ? nz - 1 : k - 1, zp = k == nz - 1 ? 0 : k + 1;
    const Rows rows = make_rows(nx, ny, i, j, k, ym, yp, zm, zp);
    const typename Codec<STORE>::T* own = fin + lbm_eoff32(n);
    const bool x_inside = i > 0 && i < nx - 1;
    if (__all_sync(__activemask(), x_inside)) Gather<STORE, false>::all(F, fin, own, map, rows, i, xm, xp);
    else Gather<STORE, true>::all(F, fin, own, map, rows, i, xm, xp);
}

#define LBM_ALL_DIRS(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17) X(18)

// v component sums: sum_s e_s[c] F[s] with zero terms dropped (SP:382-383).
template <int C, typename R>
__device__ __forceinline__ R vsum(const R* F) {
    R a = (R)0;
    bool first = true;
#pragma unroll
    for (int s = 1; s < 19; ++s) {
        const int e = C == 0 ? lbm_ex(s) : (C == 1 ? lbm_ey(s) : lbm_ez(s));
        if (e == 0) continue;
        if (first) { a = e > 0 ? F[s] : -F[s]; first = false; }
        else a = e > 0 ? a + F[s] : a - F[s];
    }
    return a;
}

// Class collision (SP:222-241): F, rho, v -> f (in place).
template <typename R, bool FORCE>
__device__ __forceinline__ void collide_sp(R* F, R r, R vx, R vy, R vz, const SpConsts<R>& C) {
    R m[19];
    mrt_moments<R>(F, m);
    const R uu = lbm_usq(vx, vy, vz);
    R meq[19];
#pragma unroll
    for (int s = 0; s < 19; ++s) meq[s] = (R)0;
    meq[0] = r; meq[3] = vx; meq[5] = vy; meq[7] = vz; meq[1] = uu;
    meq[9] = (((R)2 * vx) * vx - vy * vy) - vz * vz;
    meq[11] = vy * vy - vz * vz;
    meq[13] = vx * vy; meq[14] = vy * vz; meq[15] = vx * vz;
#pragma unroll
    for (int s = 0; s < 19; ++s) {
        const int kd = lbm_skind(s);
        if (kd == 0) continue;
        const R S = kd == 1 ? C.sv : C.so;
        m[s] = m[s] - S * (m[s] - meq[s]);
    }
    if constexpr (FORCE) {
        const R fx = C.fext[0], fy = C.fext[1], fz = C.fext[2];
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
            R g;
            if (C.guo == 0) g = a / (R)3.0 + (eu * ef) / (R)9.0;   // class (SP:236)
            else if (C.guo == 1) g = a + eu * ef;                  // scripts (TP:246)
            else g = (R)3.0 * a + (R)9.0 * (eu * ef);              // standard Guo, c_s^2 = 1/3
            G[l] = (R)lbm_w(l) * g;
        }
        R fg[19];
        mrt_moments<R>(G, fg);
#pragma unroll
        for (int s = 0; s < 19; ++s) {
            const int kd = lbm_skind(s);
            const R S = kd == 0 ? (R)0 : (kd == 1 ? C.sv : C.so);
            m[s] = m[s] + ((R)1 - (R)0.5 * S) * fg[s];
        }
    }
    mrt_back<R>(m, F);
}

// Face boundary conditions for one node on >= 1 non-periodic face
// (SP:272-370; script velocity form TP:502-506).  Faces in reference order;
// a later face overwrites what an earlier one wrote (edges, corners).
template <typename R>
__device__ __forceinline__ void apply_faces(R* F, int i, int j, int k, int n, const SpConsts<R>& C,
                                            const int32_t* __restrict__ map, const R* __restrict__ vprev) {
#pragma unroll 1
    for (int f = 0; f < 6; ++f) {
        const int bc = C.bc[f];
        if (bc == 0) continue;
        const int hi = f & 1;
        const int c = f < 2 ? i : (f < 4 ? j : k);
        const int nmax = f < 2 ? C.nx : (f < 4 ? C.ny : C.nz);
        if (c != (hi ? nmax - 1 : 0)) continue;
        R fe[19];
        if (bc == LBM_BC_PRESSURE) {
            const int inw = hi ? nmax - 2 : 1;
            const int qi = f < 2 ? inw : i, qj = (f >= 2 && f < 4) ? inw : j, qk = f >= 4 ? inw : k;
            const bool in_solid = __ldg(map + qi + C.nx * (qj + C.ny * qk)) < 0;
            R u0 = (R)0, u1 = (R)0, u2 = (R)0;
            if (!in_solid) {
                u0 = vprev[n];
                u1 = vprev[C.np + n];
                u2 = vprev[2 * C.np + n];
            }
            lbm_feq_all<R>(C.rho_bc[f], u0, u1, u2, fe);
#pragma unroll
            for (int s = 0; s < 19; ++s) F[s] = fe[s];
        } else {
            lbm_feq_all<R>((R)1.0, C.vel_bc[f][0], C.vel_bc[f][1], C.vel_bc[f][2], fe);
            if (C.bc_form == 0) {
#pragma unroll
                for (int s = 0; s < 19; ++s) F[s] = fe[s];
            } else {
#pragma unroll
                for (int s = 0; s < 19; ++s) F[s] = (fe[lbm_lr(s)] - F[lbm_lr(s)]) + fe[s];
            }
        }
    }
}

template <typename R>
__device__ __forceinline__ bool on_face(int i, int j, int k, const SpConsts<R>& C, bool pressure_only) {
    const int code = pressure_only ? LBM_BC_PRESSURE : -1;
    auto hit = [&](int f, bool at) { return at && C.bc[f] != 0 && (code < 0 || C.bc[f] == code); };
    return hit(0, i == 0) || hit(1, i == C.nx - 1) || hit(2, j == 0) || hit(3, j == C.ny - 1) || hit(4, k == 0) ||
           hit(5, k == C.nz - 1);
}

template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(256, STORE == LBM_STORE_F64 ? 1 : (FORCE ? 4 : LBM_SP_MINBLOCKS)) sp_step_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                                                      const typename Codec<STORE>::T* __restrict__ fin,
                                                      typename Codec<STORE>::T* __restrict__ fout,
                                                      const int32_t* __restrict__ map,
                                                      const uint32_t* __restrict__ coord,
                                                      typename Codec<STORE>::R* __restrict__ vprev,
                                                      typename Codec<STORE>::R* __restrict__ rho_out,
                                                      typename Codec<STORE>::R* __restrict__ v_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
    const int64_t np = C.np;

    R F[19];
    gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k);

    // Face nodes are rare; warps without one skip the branch uniformly.
    bool face = false;
    if (C.any_bc) {
        face = on_face(i, j, k, C, false);
        if (face) apply_faces<R>(F, i, j, k, n, C, map, vprev);
    }

    // macros (SP:376-388)
    R r = F[0];
#pragma unroll
    for (int s = 1; s < 19; ++s) r = r + F[s];
    R vx = vsum<0>(F), vy = vsum<1>(F), vz = vsum<2>(F);
    vx = vx / r;
    vy = vy / r;
    vz = vz / r;
    if constexpr (FORCE) {
        vx = vx + C.fhalf[0] / r;
        vy = vy + C.fhalf[1] / r;
        vz = vz + C.fhalf[2] / r;
    }
    if (face && C.any_pressure && on_face(i, j, k, C, true)) {
        vprev[n] = vx;
        vprev[np + n] = vy;
        vprev[2 * np + n] = vz;
    }
    if constexpr (MACROS) {
        rho_out[n] = r;
        v_out[n] = vx;
        v_out[np + n] = vy;
        v_out[2 * np + n] = vz;
    }

    collide_sp<R, FORCE>(F, r, vx, vy, vz, C);
    typename Cd::T* out = fout + lbm_eoff32(n);
#define LBM_S(S) out[32 * S] = Cd::template enc<S>(F[S]);
    LBM_S(0) LBM_ALL_DIRS(LBM_S)
#undef LBM_S
}

// Initial populations: F = feq(rho, v), then one collision with (rho, v)
// (init SP:160-170 followed by the first step's colission).
template <int STORE, bool FORCE>
__global__ void sp_init_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                               typename Codec<STORE>::T* __restrict__ fout, const float* __restrict__ rho_in,
                               const float* __restrict__ v_in, typename Codec<STORE>::R* __restrict__ vprev) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const int64_t np = C.np;
    R r = (R)1.0, vx = (R)0, vy = (R)0, vz = (R)0;
    if (rho_in) {
        r = (R)rho_in[n];
        vx = (R)v_in[n];
        vy = (R)v_in[np + n];
        vz = (R)v_in[2 * np + n];
    }
    R F[19];
    lbm_feq_all<R>(r, vx, vy, vz, F);
    vprev[n] = vx;
    vprev[np + n] = vy;
    vprev[2 * np + n] = vz;
    collide_sp<R, FORCE>(F, r, vx, vy, vz, C);
    typename Cd::T* out = fout + lbm_eoff32(n);
#define LBM_S(S) out[32 * S] = Cd::template enc<S>(F[S]);
    LBM_S(0) LBM_ALL_DIRS(LBM_S)
#undef LBM_S
}

// Pure pull-stream (identity collision, no faces): the permutation check.
__global__ void sp_gather_kernel(const __grid_constant__ SpConsts<float> C, const float* __restrict__ fin,
                                 float* __restrict__ fout, const int32_t* __restrict__ map,
                                 const uint32_t* __restrict__ coord) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = coord[n];
    float F[19];
    gather_node<LBM_STORE_F32>(F, fin, map, n, C.nx, C.ny, C.nz, lbm_pi(pc), lbm_pj(pc), lbm_pk(pc));
    float* out = fout + lbm_eoff32(n);
#pragma unroll
    for (int s = 0; s < 19; ++s) out[32 * s] = F[s];
}

template <int STORE, bool FORCE, bool MACROS>
int launch_step(LbmHandle* h, const SpConsts<typename Codec<STORE>::R>& C, int grid) {
    using T = typename Codec<STORE>::T;
    using R = typename Codec<STORE>::R;
    const T* fin = (const T*)h->d_f[h->cur];
    T* fout = (T*)h->d_f[h->cur ^ 1];
    sp_step_kernel<STORE, FORCE, MACROS><<<grid, h->block, 0, h->stream>>>(
        C, fin, fout, h->d_map, h->d_coord, (R*)h->d_vprev, (R*)h->d_rho, (R*)h->d_v);
    h->cur ^= 1;
    return lbm_cuda_check(h, cudaGetLastError(), "sp_step_kernel launch");
}

template <int STORE>
int run_steps(LbmHandle* h, int32_t n, bool macros_last) {
    using R = typename Codec<STORE>::R;
    const SpConsts<R> C = sp_make_consts<R>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    for (int32_t it = 0; it < n; ++it) {
        const bool mac = macros_last && it == n - 1;
        int rc;
        if (h->force) rc = mac ? launch_step<STORE, true, true>(h, C, grid) : launch_step<STORE, true, false>(h, C, grid);
        else rc = mac ? launch_step<STORE, false, true>(h, C, grid) : launch_step<STORE, false, false>(h, C, grid);
        if (rc) return rc;
    }
    return LBM_OK;
}

template <int STORE>
int run_init(LbmHandle* h, const float* rho, const float* v) {
    using T = typename Codec<STORE>::T;
    using R = typename Codec<STORE>::R;
    const SpConsts<R> C = sp_make_consts<R>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    T* fout = (T*)h->d_f[h->cur];
    if (h->force) sp_init_kernel<STORE, true><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev);
    else sp_init_kernel<STORE, false><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev);
    return lbm_cuda_check(h, cudaGetLastError(), "sp_init_kernel launch");
}

}  // namespace

template <typename R>
SpConsts<R> sp_make_consts(const LbmHandle* h) {
    const LbmParams& p = h->p;
    SpConsts<R> C{};
    C.nx = p.nx; C.ny = p.ny; C.nz = p.nz;
    C.n_fluid = h->n_fluid;
    C.np = h->np;
    C.any_bc = 0; C.any_pressure = 0;
    for (int f = 0; f < 6; ++f) {
        C.bc[f] = p.bc[f];
        C.any_bc |= p.bc[f] != 0;
        C.any_pressure |= p.bc[f] == LBM_BC_PRESSURE;
        C.rho_bc[f] = (R)p.rho_bc[f];
        for (int c = 0; c < 3; ++c) C.vel_bc[f][c] = (R)p.vel_bc[f][c];
    }
    C.bc_form = p.bc_form;
    C.guo = p.guo_convention;
    // init_simulation (SP:126-131); the product keeps Python's FP64 for tau, s_v, s_other
    // and rounds once, as Taichi does when it stores them into the f32 S_dig field.
    const double tau = p.visc_convention == 0 ? p.niu / 3.0 + 0.5 : 3.0 * p.niu + 0.5;
    const double sv = 1.0 / tau;
    const double so = 8.0 * (2.0 - sv) / (8.0 - sv);
    C.sv = (R)sv;
    C.so = (R)so;
    for (int c = 0; c < 3; ++c) {
        C.fext[c] = (R)p.force[c];
        C.fhalf[c] = C.fext[c] / (R)2;
    }
    return C;
}
template SpConsts<float> sp_make_consts<float>(const LbmHandle*);
template SpConsts<double> sp_make_consts<double>(const LbmHandle*);

int sp_launch_steps(LbmHandle* h, int32_t n, bool macros_last) {
    switch (h->p.storage) {
    case LBM_STORE_F32: return run_steps<LBM_STORE_F32>(h, n, macros_last);
    case LBM_STORE_F16_DEV: return run_steps<LBM_STORE_F16_DEV>(h, n, macros_last);
    case LBM_STORE_BF16_DEV: return run_steps<LBM_STORE_BF16_DEV>(h, n, macros_last);
    case LBM_STORE_F64: return run_steps<LBM_STORE_F64>(h, n, macros_last);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}

int sp_launch_init(LbmHandle* h, const void* rho_nodes, const void* v_nodes) {
    const float* r = (const float*)rho_nodes;
    const float* v = (const float*)v_nodes;
    switch (h->p.storage) {
    case LBM_STORE_F32: return run_init<LBM_STORE_F32>(h, r, v);
    case LBM_STORE_F16_DEV: return run_init<LBM_STORE_F16_DEV>(h, r, v);
    case LBM_STORE_BF16_DEV: return run_init<LBM_STORE_BF16_DEV>(h, r, v);
    case LBM_STORE_F64: return run_init<LBM_STORE_F64>(h, r, v);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}

int sp_launch_debug_stream(LbmHandle* h, const float* d_in, float* d_out) {
    const SpConsts<float> C = sp_make_consts<float>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    sp_gather_kernel<<<grid, h->block, 0, h->stream>>>(C, d_in, d_out, h->d_map, h->d_coord);
    return lbm_cuda_check(h, cudaGetLastError(), "sp_gather_kernel launch");
}
