// Device building blocks shared by the fused step kernels: pull gather over
// the compacted node list, face boundary conditions, macroscopic sums and the
// single-phase MRT collision.  Paths: SP = Single_phase/LBM_3D_SinglePhase_Solver.py,
// TP = 2phase/lbm_solver_3d_2phase_sparse.py (taichi_LBM3D tree).
#pragma once
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbmk {

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

// Node index of the pull source x - e_S of a node (or -1 when that cell is solid).
template <int S, bool XWRAP>
__device__ __forceinline__ int pull_source(const int32_t* __restrict__ map, const Rows& rows, int i, int xm, int xp) {
    constexpr int ex = lbm_ex(S), ey = lbm_ey(S), ez = lbm_ez(S);
    // source is x - e_S: row index 0 holds y-1 (used when ey = +1)
    const int row = rows.r[1 - ey][1 - ez];
    if constexpr (XWRAP) {
        const int x = ex > 0 ? xm : (ex < 0 ? xp : i);
        return __ldg(map + (row - i + x));
    } else {
        return __ldg(map + row - ex);
    }
}

#ifdef LBM_DEBUG
// Debug builds (-DLBM_DEBUG): the first failed index check is recorded here
// (1 = node coordinates outside the lattice, 2 = a map entry beyond the
// fluid-node count) and read back by the host after the step; the offending
// access is skipped.  One copy per translation unit; the single-phase step
// (lbm_sp.cu) sets the node limit and reads the flag; elsewhere the limit
// stays 0 and the check is off.
static __device__ int g_lbm_debug;
static __device__ int g_lbm_debug_nlimit;
__device__ __forceinline__ void lbm_debug_fail(int code) { atomicCAS(&g_lbm_debug, 0, code); }
#endif

template <typename R>
__host__ __device__ __forceinline__ LbmRef<R> sp_ref(const SpConsts<R>& C) {
    LbmRef<R> r;
    r.a = C.ref_a;
    r.b = C.ref_b;
    return r;
}

// RHOREF codecs: the reference density at the node's x (ri) and the profile
// (a + b x) for the sources: x - e_x, or the wrapped x on x-face warps.
template <typename R>
struct RefX {
    R ri, a, b;
};
template <int STORE>
__device__ __forceinline__ RefX<typename Codec<STORE>::R> ref_x(const LbmRef<typename Codec<STORE>::R>& ref, int i) {
    RefX<typename Codec<STORE>::R> x{};
    if constexpr (Codec<STORE>::RHOREF) {
        x.a = ref.a;
        x.b = ref.b;
        x.ri = lbm_ref_at(ref, i);
    }
    return x;
}

template <int STORE, bool XWRAP>
struct Gather {
    using Cd = Codec<STORE>;
    using T = typename Cd::T;
    using R = typename Cd::R;
    template <int S>
    static __device__ __forceinline__ void one(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* __restrict__ map, const Rows& rows, int i, int xm,
                                               int xp, const RefX<R>& rx) {
#ifdef LBM_DEBUG
        int src = pull_source<S, XWRAP>(map, rows, i, xm, xp);
        if (g_lbm_debug_nlimit > 0 && src >= g_lbm_debug_nlimit) {
            lbm_debug_fail(2);
            src = -1;
        }
#else
        const int src = pull_source<S, XWRAP>(map, rows, i, xm, xp);
#endif
        load_pulled<S>(F, src, fin, own, rx, XWRAP ? (lbm_ex(S) > 0 ? xm : (lbm_ex(S) < 0 ? xp : i)) : i - lbm_ex(S));
    }
    // F[S] from the pull source node src (or the own LR[S] slot when src < 0):
    // one load from the selected address (+3% FP32, +4% FP32 deviation form on
    // the 256^3 pack against two predicated loads).  RHOREF: plus w_S times the
    // reference density at the source's x, xs (the node's own x for bounce-back).
    template <int S>
    static __device__ __forceinline__ void load_pulled(R* F, int src, const T* __restrict__ fin,
                                                       const T* __restrict__ own, const RefX<R>& rx, int xs) {
        const T* a = src >= 0 ? fin + lbm_eoff32(src) + 32 * S : own + 32 * lbm_lr(S);
        F[S] = Cd::template dec<S>(*a);
        if constexpr (Cd::RHOREF) {
            R rs = rx.ri;
            if constexpr (lbm_ex(S) != 0) {
                if constexpr (XWRAP) rs = lbm_fma<R>(rx.b, (R)xs, rx.a);
                else rs = lbm_ex(S) > 0 ? rx.ri - rx.b : rx.ri + rx.b;
            }
            F[S] = lbm_fma<R>((R)lbm_w(S), src >= 0 ? rs : rx.ri, F[S]);
        }
    }
    static __device__ __forceinline__ void all(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* __restrict__ map, const Rows& rows, int i, int xm,
                                               int xp, const RefX<R>& rx) {
        F[0] = Cd::template dec<0>(own[0]);
        if constexpr (Cd::RHOREF) F[0] = lbm_fma<R>((R)lbm_w(0), rx.ri, F[0]);
#define LBM_G(S) one<S>(F, fin, own, map, rows, i, xm, xp, rx);
        LBM_G(1) LBM_G(2) LBM_G(3) LBM_G(4) LBM_G(5) LBM_G(6) LBM_G(7) LBM_G(8) LBM_G(9)
        LBM_G(10) LBM_G(11) LBM_G(12) LBM_G(13) LBM_G(14) LBM_G(15) LBM_G(16) LBM_G(17) LBM_G(18)
#undef LBM_G
    }
};

// Gather F for node n; warps with no lane on an x face take the immediate-offset path.
template <int STORE>
__device__ __forceinline__ void gather_node(typename Codec<STORE>::R* F, const typename Codec<STORE>::T* __restrict__ fin,
                                            const int32_t* __restrict__ map, int n, int nx, int ny, int nz, int i, int j,
                                            int k,
                                            const LbmRef<typename Codec<STORE>::R>& ref = LbmRef<typename Codec<STORE>::R>()) {
    const int xm = i == 0 ? nx - 1 : i - 1, xp = i == nx - 1 ? 0 : i + 1;
    const int ym = j == 0 ? ny - 1 : j - 1, yp = j == ny - 1 ? 0 : j + 1;
    const int zm = k == 0 ? nz - 1 : k - 1, zp = k == nz - 1 ? 0 : k + 1;
    const Rows rows = make_rows(nx, ny, i, j, k, ym, yp, zm, zp);
    const typename Codec<STORE>::T* own = fin + lbm_eoff32(n);
    const auto rx = ref_x<STORE>(ref, i);
    const bool x_inside = i > 0 && i < nx - 1;
    if (__all_sync(__activemask(), x_inside)) Gather<STORE, false>::all(F, fin, own, map, rows, i, xm, xp, rx);
    else Gather<STORE, true>::all(F, fin, own, map, rows, i, xm, xp, rx);
}

// Gather through a shared-memory copy of the map: planes pz = 0, 1, 2 hold
// source z = k - 1, k, k + 1 (wrapped), each a block of whole x rows starting
// one row before the node's; b[pz] is the node's own cell in plane pz (row
// offset and the plane's alignment shift included), so the source x - e_S sits
// at b[1 - ez] - ey nx - ex (x faces: wrapped x).
template <int STORE, bool XWRAP>
struct GatherS {
    using G = Gather<STORE, XWRAP>;
    using T = typename G::T;
    using R = typename G::R;
    template <int S>
    static __device__ __forceinline__ void one(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* sm, const int (&b)[3], int nx, int i, int xm, int xp,
                                               const RefX<R>& rx) {
        constexpr int ex = lbm_ex(S), ey = lbm_ey(S), ez = lbm_ez(S);
        int idx = b[1 - ez] - ey * nx;
        if constexpr (XWRAP) idx += (ex > 0 ? xm : (ex < 0 ? xp : i)) - i;
        else idx -= ex;
#ifdef LBM_DEBUG
        int src = sm[idx];
        if (g_lbm_debug_nlimit > 0 && src >= g_lbm_debug_nlimit) {
            lbm_debug_fail(2);
            src = -1;
        }
#else
        const int src = sm[idx];
#endif
        G::template load_pulled<S>(F, src, fin, own, rx, XWRAP ? (ex > 0 ? xm : (ex < 0 ? xp : i)) : i - ex);
    }
    static __device__ __forceinline__ void all(R* F, const T* __restrict__ fin, const T* __restrict__ own,
                                               const int32_t* sm, const int (&b)[3], int nx, int i, int xm, int xp,
                                               const RefX<R>& rx) {
        F[0] = Codec<STORE>::template dec<0>(own[0]);
        if constexpr (Codec<STORE>::RHOREF) F[0] = lbm_fma<R>((R)lbm_w(0), rx.ri, F[0]);
#define LBM_G(S) one<S>(F, fin, own, sm, b, nx, i, xm, xp, rx);
        LBM_G(1) LBM_G(2) LBM_G(3) LBM_G(4) LBM_G(5) LBM_G(6) LBM_G(7) LBM_G(8) LBM_G(9)
        LBM_G(10) LBM_G(11) LBM_G(12) LBM_G(13) LBM_G(14) LBM_G(15) LBM_G(16) LBM_G(17) LBM_G(18)
#undef LBM_G
    }
};

template <int STORE>
__device__ __forceinline__ void gather_node_smem(typename Codec<STORE>::R* F,
                                                 const typename Codec<STORE>::T* __restrict__ fin, const int32_t* sm,
                                                 const int (&b)[3], int n, int nx, int i,
                                                 const LbmRef<typename Codec<STORE>::R>& ref) {
    const int xm = i == 0 ? nx - 1 : i - 1, xp = i == nx - 1 ? 0 : i + 1;
    const typename Codec<STORE>::T* own = fin + lbm_eoff32(n);
    const auto rx = ref_x<STORE>(ref, i);
    const bool x_inside = i > 0 && i < nx - 1;
    if (__all_sync(__activemask(), x_inside)) GatherS<STORE, false>::all(F, fin, own, sm, b, nx, i, xm, xp, rx);
    else GatherS<STORE, true>::all(F, fin, own, sm, b, nx, i, xm, xp, rx);
}

#define LBM_ALL_DIRS(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17) X(18)

// Store node n's post-collision populations.  RHOREF codecs store them
// relative to the reference density at the node's x (g = f' - w ref), rounded
// stochastically with the bits of (n, seed) (LBM_SR).
template <int STORE>
__device__ __forceinline__ void store_node(const typename Codec<STORE>::R* F, typename Codec<STORE>::T* __restrict__ fout,
                                           int n, typename Codec<STORE>::R ref_own, uint32_t seed) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    typename Cd::T* out = fout + lbm_eoff32(n);
    if constexpr (Cd::RHOREF) {
#if LBM_SR
        const uint32_t h = lbm_sr_hash((uint32_t)n, seed);
#define LBM_S(S) out[32 * S] = Cd::template enc_sr<S>(lbm_fma<R>(-(R)lbm_w(S), ref_own, F[S]), h);
#else
        (void)seed;
#define LBM_S(S) out[32 * S] = Cd::template enc<S>(lbm_fma<R>(-(R)lbm_w(S), ref_own, F[S]));
#endif
        LBM_S(0) LBM_ALL_DIRS(LBM_S)
#undef LBM_S
    } else {
        (void)ref_own;
        (void)seed;
#define LBM_S(S) out[32 * S] = Cd::template enc<S>(F[S]);
        LBM_S(0) LBM_ALL_DIRS(LBM_S)
#undef LBM_S
    }
}

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

// Class collision (SP:222-241): F, rho, v -> f (in place).  In deviation form
// F holds f - w and r is rho - 1 (moment 0 of M (f - w)).
// FAST (deviation-form kernels): pair-form transforms and FMA relaxation; the
// reference-arithmetic kernels keep the term-by-term order (FAST = false).
template <typename R, bool FORCE, bool FAST = false>
__device__ __forceinline__ void collide_sp(R* F, R r, R vx, R vy, R vz, const SpConsts<R>& C) {
    R m[19];
    if constexpr (FAST) mrt_moments_fast<R>(F, m);
    else mrt_moments<R>(F, m);
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
        if constexpr (FAST) m[s] = lbm_fma<R>(S, meq[s] - m[s], m[s]);
        else m[s] = m[s] - S * (m[s] - meq[s]);
    }
    if constexpr (FORCE && FAST) {
        // M (w o g) in closed form, from sum_l M_rl w_l, sum_l M_rl w_l e_l and
        // sum_l M_rl w_l e_l e_l^T of this M (checked in tests/test_host_tables.py):
        // moment 0: (gd/3 - gc) u.F,
        // moment 1: 2/9 gd u.F, moments 3, 5, 7: gc F / 3, moment 9:
        // gd (4 ux Fx - 2 uy Fy - 2 uz Fz) / 9, moment 11: 2/9 gd (uy Fy - uz Fz),
        // moments 13, 14, 15: gd (ua Fb + ub Fa) / 9; the others vanish.  Moments
        // 0, 3, 5, 7 are conserved (S = 0); 1, 9, 11, 13-15 relax with s_v.
        const R fx = C.fext[0], fy = C.fext[1], fz = C.fext[2];
        const R gc = C.gc, gd = C.gd;
        const R ksv = (R)1 - (R)0.5 * C.sv;
        const R uf = lbm_fma<R>(vz, fz, lbm_fma<R>(vy, fy, vx * fx));
        const R d9 = gd * (R)(1.0 / 9.0);
        m[0] = lbm_fma<R>(gd * (R)(1.0 / 3.0) - gc, uf, m[0]);
        m[1] = lbm_fma<R>(ksv * (R)2 * d9, uf, m[1]);
        const R c3 = gc * (R)(1.0 / 3.0);
        m[3] = lbm_fma<R>(c3, fx, m[3]);
        m[5] = lbm_fma<R>(c3, fy, m[5]);
        m[7] = lbm_fma<R>(c3, fz, m[7]);
        const R kd9 = ksv * d9;
        m[9] = lbm_fma<R>(kd9, (R)4 * (vx * fx) - (R)2 * lbm_fma<R>(vy, fy, vz * fz), m[9]);
        m[11] = lbm_fma<R>(kd9 * (R)2, lbm_fma<R>(vy, fy, -(vz * fz)), m[11]);
        m[13] = lbm_fma<R>(kd9, lbm_fma<R>(vx, fy, vy * fx), m[13]);
        m[14] = lbm_fma<R>(kd9, lbm_fma<R>(vy, fz, vz * fy), m[14]);
        m[15] = lbm_fma<R>(kd9, lbm_fma<R>(vx, fz, vz * fx), m[15]);
    } else if constexpr (FORCE) {
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
    if constexpr (FAST) mrt_back_fast<R>(m, F);
    else mrt_back<R>(m, F);
}

// Face boundary conditions for one node on >= 1 non-periodic face
// (SP:272-370; script velocity form TP:502-506).  Faces in reference order;
// a later face overwrites what an earlier one wrote (edges, corners).
template <typename R, bool DEV = false>
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
            if constexpr (DEV) lbm_feq_dev_all<R>(C.rho_bc_dev[f], u0, u1, u2, fe);
            else lbm_feq_all<R>(C.rho_bc[f], u0, u1, u2, fe);
#pragma unroll
            for (int s = 0; s < 19; ++s) F[s] = fe[s];
        } else {
            // in deviation form the in-place form keeps its shape: the w terms cancel
            if constexpr (DEV) lbm_feq_dev_all<R>((R)0, C.vel_bc[f][0], C.vel_bc[f][1], C.vel_bc[f][2], fe);
            else lbm_feq_all<R>((R)1.0, C.vel_bc[f][0], C.vel_bc[f][1], C.vel_bc[f][2], fe);
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


}  // namespace lbmk
