// D3Q19 tables, equilibrium and population storage codecs shared by the
// fused kernels.  Arithmetic is written term by term in the order of the
// reference's Taichi expressions (paths inside the taichi_LBM3D tree):
//   SP = Single_phase/LBM_3D_SinglePhase_Solver.py
//   TP = 2phase/lbm_solver_3d_2phase_sparse.py
// and the library is compiled with -fmad=false, so that no multiply-add is
// fused unless written as lbm_fma() on an exact product.  Together with IEEE
// division this makes the FP32 kernels reproduce the reference arithmetic
// bit for bit (terms with an exactly-zero coefficient are dropped, which does
// not change a non-zero partial sum).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/lbm_gb300.h"

#define LBM_HD __host__ __device__ __forceinline__

// e, w, LR: SP:183-197, SP:85.
__host__ __device__ constexpr int lbm_ex(int s) {
    return (s == 1 || s == 7 || s == 9 || s == 11 || s == 13) ? 1
         : (s == 2 || s == 8 || s == 10 || s == 12 || s == 14) ? -1 : 0;
}
__host__ __device__ constexpr int lbm_ey(int s) {
    return (s == 3 || s == 7 || s == 10 || s == 15 || s == 17) ? 1
         : (s == 4 || s == 8 || s == 9 || s == 16 || s == 18) ? -1 : 0;
}
__host__ __device__ constexpr int lbm_ez(int s) {
    return (s == 5 || s == 11 || s == 14 || s == 15 || s == 18) ? 1
         : (s == 6 || s == 12 || s == 13 || s == 16 || s == 17) ? -1 : 0;
}
__host__ __device__ constexpr int lbm_lr(int s) { return s == 0 ? 0 : ((s & 1) ? s + 1 : s - 1); }
__host__ __device__ constexpr double lbm_w(int s) { return s == 0 ? 1.0 / 3.0 : (s <= 6 ? 1.0 / 18.0 : 1.0 / 36.0); }
// S_dig pattern (SP:131): 0 conserved, 1 s_v, 2 s_other.
__host__ __device__ constexpr int lbm_skind(int s) {
    return (s == 0 || s == 3 || s == 5 || s == 7) ? 0 : ((s == 4 || s == 6 || s == 8 || s >= 16) ? 2 : 1);
}

template <typename R>
LBM_HD R lbm_fma(R a, R b, R c);
template <>
LBM_HD float lbm_fma<float>(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
template <>
LBM_HD double lbm_fma<double>(double a, double b, double c) {
#ifdef __CUDA_ARCH__
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

#include "mrt_gen.cuh"

// e_s . u with the zero components dropped (SP:154 e[k].dot(u)).
template <int S, typename R>
LBM_HD R lbm_edot(R u0, R u1, R u2) {
    constexpr int ex = lbm_ex(S), ey = lbm_ey(S), ez = lbm_ez(S);
    if constexpr (ex == 0 && ey == 0 && ez == 0) {
        return (R)0;
    } else if constexpr (ex != 0) {
        R a = ex > 0 ? u0 : -u0;
        if constexpr (ey != 0) a = ey > 0 ? a + u1 : a - u1;
        if constexpr (ez != 0) a = ez > 0 ? a + u2 : a - u2;
        return a;
    } else if constexpr (ey != 0) {
        R a = ey > 0 ? u1 : -u1;
        if constexpr (ez != 0) a = ez > 0 ? a + u2 : a - u2;
        return a;
    } else {
        return ez > 0 ? u2 : -u2;
    }
}

// feq (SP:152-158): w*rho*(1.0+3.0*eu+4.5*eu*eu-1.5*uv), uv = u.u precomputed.
template <int S, typename R>
LBM_HD R lbm_feq(R rho, R u0, R u1, R u2, R uv) {
    R eu = lbm_edot<S, R>(u0, u1, u2);
    R t = (R)1.0 + (R)3.0 * eu;
    t = t + ((R)4.5 * eu) * eu;
    t = t - (R)1.5 * uv;
    return ((R)lbm_w(S) * rho) * t;
}

template <typename R>
LBM_HD R lbm_usq(R u0, R u1, R u2) {
    R a = u0 * u0;
    a = a + u1 * u1;
    return a + u2 * u2;
}

// Runtime-direction feq (face boundary conditions).
template <typename R>
__device__ __forceinline__ void lbm_feq_all(R rho, R u0, R u1, R u2, R* out) {
    const R uv = lbm_usq(u0, u1, u2);
#define LBM_FQ(S) out[S] = lbm_feq<S, R>(rho, u0, u1, u2, uv);
    LBM_FQ(0) LBM_FQ(1) LBM_FQ(2) LBM_FQ(3) LBM_FQ(4) LBM_FQ(5) LBM_FQ(6) LBM_FQ(7) LBM_FQ(8) LBM_FQ(9)
    LBM_FQ(10) LBM_FQ(11) LBM_FQ(12) LBM_FQ(13) LBM_FQ(14) LBM_FQ(15) LBM_FQ(16) LBM_FQ(17) LBM_FQ(18)
#undef LBM_FQ
}

// ---------------------------------------------------------------- storage
// Population codecs: Codec<STORE>::T is the stored element type, R the compute
// type.  DEV codecs compute in deviation form: the kernel works on
// f' = f - w and rho' = rho - 1 (the transforms are linear and M w is the unit
// vector of moment 0, so only moment 0 and the macroscopic density change),
// which keeps the small flow signal out of the rounding of f ~ w.  RHOREF
// codecs (16-bit) store g = f' - w rho'_ref(x) with a fixed reference density
// rho'_ref that every reader can compute from the cell's x coordinate (LbmRef:
// the linear profile between two fixed-pressure x faces, else 0), so what is
// left in g is the local density departure, the velocity and non-equilibrium
// part, which 16-bit storage can resolve (FP16 scaled by 2^16: |g| from ~1e-9
// to 1 keeps 11 significant bits) without any per-node side array.
//
// Encoding rounds stochastically (LBM_SR = 1, the default): random bits below
// the kept mantissa are added to the FP32 pattern before it is truncated, so a
// stored value is unbiased.  Rounding to nearest stalls slow steady flows, whose
// per-step change of a population is a few 16-bit ulps (a 16-cell channel
// stalled 3.8% off the parabola in FP16, 31% in BF16).  The random bits come
// from a hash of (node, step), one 32-bit word per node and a multiplicative
// spread per direction, so runs are deterministic.
#ifndef LBM_SR
#define LBM_SR 1
#endif

template <typename R>
struct LbmRef {
    R a = (R)0, b = (R)0;   // rho'_ref(i) = a + b i
};
template <typename R>
__device__ __forceinline__ R lbm_ref_at(const LbmRef<R>& r, int i) {
    return lbm_fma<R>(r.b, (R)i, r.a);
}

// 32 random bits per (node, step) (a xor-multiply avalanche of both).
__device__ __forceinline__ uint32_t lbm_sr_hash(uint32_t n, uint32_t seed) {
    uint32_t x = n * 0x9E3779B1u ^ (seed * 0x85EBCA77u + 0x632BE5ABu);
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
// Direction S's bits: an odd multiplier per direction, top bits kept.
template <int S>
__device__ __forceinline__ uint32_t lbm_sr_bits(uint32_t h) {
    return h * (0x2545F491u + 2u * 0x9E37u * (uint32_t)S);
}

template <int STORE> struct Codec;
template <> struct Codec<LBM_STORE_F32> {
    using T = float; using R = float;
    static constexpr bool DEV = false, RHOREF = false;
    template <int S> static __device__ __forceinline__ R dec(T x) { return x; }
    template <int S> static __device__ __forceinline__ T enc(R f) { return f; }
};
template <> struct Codec<LBM_STORE_F64> {
    using T = double; using R = double;
    static constexpr bool DEV = false, RHOREF = false;
    template <int S> static __device__ __forceinline__ R dec(T x) { return x; }
    template <int S> static __device__ __forceinline__ T enc(R f) { return f; }
};
template <> struct Codec<LBM_STORE_F32_DEV> {
    using T = float; using R = float;
    static constexpr bool DEV = true, RHOREF = false;
    template <int S> static __device__ __forceinline__ R dec(T x) { return x; }
    template <int S> static __device__ __forceinline__ T enc(R f) { return f; }
};
template <> struct Codec<LBM_STORE_F16_DEV> {
    using T = __half; using R = float;
    static constexpr bool DEV = true, RHOREF = true;
    template <int S> static __device__ __forceinline__ R dec(T x) { return __half2float(x) * (1.0f / 65536.0f); }
    template <int S> static __device__ __forceinline__ T enc(R g) { return __float2half_rn(g * 65536.0f); }
    // 13 bits below the FP16 mantissa (exact for FP16 normals; FP16
    // subnormals, |g| < 1e-9, keep a bias below one of their ulps)
    template <int S> static __device__ __forceinline__ T enc_sr(R g, uint32_t h) {
        const uint32_t u = __float_as_uint(g * 65536.0f) + (lbm_sr_bits<S>(h) >> 19);
        return __float2half_rz(__uint_as_float(u));
    }
};
template <> struct Codec<LBM_STORE_BF16_DEV> {
    using T = __nv_bfloat16; using R = float;
    static constexpr bool DEV = true, RHOREF = true;
    template <int S> static __device__ __forceinline__ R dec(T x) { return __bfloat162float(x); }
    template <int S> static __device__ __forceinline__ T enc(R g) { return __float2bfloat16_rn(g); }
    template <int S> static __device__ __forceinline__ T enc_sr(R g, uint32_t h) {
        const uint32_t u = __float_as_uint(g) + (lbm_sr_bits<S>(h) >> 16);
        return __float2bfloat16_rz(__uint_as_float(u));
    }
};

// feq_S(rho, u) - w_S with rho = 1 + rho' (deviation form of lbm_feq).
template <int S, typename R>
LBM_HD R lbm_feq_dev(R rho_dev, R u0, R u1, R u2, R uv) {
    R eu = lbm_edot<S, R>(u0, u1, u2);
    R t = (R)3.0 * eu + ((R)4.5 * eu) * eu;
    t = t - (R)1.5 * uv;
    return (R)lbm_w(S) * (rho_dev + ((R)1 + rho_dev) * t);
}

template <typename R>
__device__ __forceinline__ void lbm_feq_dev_all(R rho_dev, R u0, R u1, R u2, R* out) {
    const R uv = lbm_usq(u0, u1, u2);
#define LBM_FQ(S) out[S] = lbm_feq_dev<S, R>(rho_dev, u0, u1, u2, uv);
    LBM_FQ(0) LBM_FQ(1) LBM_FQ(2) LBM_FQ(3) LBM_FQ(4) LBM_FQ(5) LBM_FQ(6) LBM_FQ(7) LBM_FQ(8) LBM_FQ(9)
    LBM_FQ(10) LBM_FQ(11) LBM_FQ(12) LBM_FQ(13) LBM_FQ(14) LBM_FQ(15) LBM_FQ(16) LBM_FQ(17) LBM_FQ(18)
#undef LBM_FQ
}

// Population layout "AoSoA-32": nodes in chunks of 32; within a chunk the 19
// directions follow one another, 32 consecutive nodes each.  Element (n, s) is
// at lbm_eoff(n) + 32*s, so a warp's 32 nodes touch one 128 B (FP32) segment per
// direction and a thread addresses all 19 of its slots with immediate offsets.
LBM_HD int64_t lbm_eoff(int64_t n) { return n + (n >> 5) * 576; }
LBM_HD int64_t lbm_pidx(int64_t n, int s) { return lbm_eoff(n) + 32 * s; }
__device__ __forceinline__ int lbm_eoff32(int n) { return n + (n >> 5) * 576; }

// Lattice coordinates of a fluid node, packed i | j<<11 | k<<22.
LBM_HD uint32_t lbm_pack(int i, int j, int k) { return (uint32_t)i | ((uint32_t)j << 11) | ((uint32_t)k << 22); }
LBM_HD int lbm_pi(uint32_t p) { return (int)(p & 2047u); }
LBM_HD int lbm_pj(uint32_t p) { return (int)((p >> 11) & 2047u); }
LBM_HD int lbm_pk(uint32_t p) { return (int)(p >> 22); }
