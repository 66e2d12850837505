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
// Memory layout (HBM): populations in AoSoA-32 chunks (element (n, s) at
// n + (n >> 5) * 576 + 32 s, lbm_common.cuh) in two buffers (ping-pong),
// np = n_fluid padded to 64; dense int32 map cell -> node (or -1 for solid),
// kept L2-resident by a persisting access-policy window (lbm_capi.cu); packed
// node coordinates.  Per node and step the kernel moves 19 loads + 19 stores
// of populations (152 B in FP32, 76 B in 16-bit storage), 4 B of coordinates
// and the neighbour map rows (L1/L2 hits).
//
// Consecutive steps use programmatic dependent launch: a step's CTAs load their
// coordinates while the previous step drains, then wait for it (+1.5% on the
// 256^3 pack).  Measured and rejected on the same pack: a persistent
// grid-stride loop with the next node's coordinates prefetched (24.1k against
// 33.2k MLUPS: the block-ordered launch keeps the active node window compact
// in L2) and cp.async prefetch of the next node's 19 populations into shared
// memory (17.1k: per-element 4-byte copies stall on the MIO queue).
#include <cuda_runtime.h>

#include "lbm_common.cuh"
#include "lbm_internal.h"
#include "lbm_kernels.cuh"

// Resident 256-thread CTAs per SM requested for the step kernel (caps
// registers at 65536 / (256 * n)).  The reference-arithmetic FP32 kernel is
// fastest at 6 (40 registers), 4 with the dense Guo forcing; the
// deviation-form kernels, whose pair-form transforms keep more values live,
// spill at 6 and are fastest at 5, forced or not (measured on the 256^3 pack:
// unforced f32dev +4%, FP16 +8%, BF16 +13% over 6; forced +1%, +7%, +4%
// over 4).
#ifndef LBM_SP_MINBLOCKS
#define LBM_SP_MINBLOCKS 6
#endif
#ifndef LBM_SP_MINBLOCKS_DEV
#define LBM_SP_MINBLOCKS_DEV 5
#endif
// Programmatic dependent launch of consecutive steps: each step's CTAs may
// become resident while the previous step drains and wait (griddepcontrol)
// before touching populations or boundary state.  0 = plain stream order.
#ifndef LBM_SP_PDL
#define LBM_SP_PDL 1
#endif

namespace {
using namespace lbmk;

// Everything after the gather: faces, macros, collision and store of node n.
template <int STORE, bool FORCE, bool MACROS>
__device__ __forceinline__ void sp_finish_node(typename Codec<STORE>::R* F, int n, int i, int j, int k,
                                               const SpConsts<typename Codec<STORE>::R>& C,
                                               typename Codec<STORE>::T* __restrict__ fout,
                                               const int32_t* __restrict__ map,
                                               typename Codec<STORE>::R* __restrict__ vprev,
                                               typename Codec<STORE>::R* __restrict__ rho_out,
                                               typename Codec<STORE>::R* __restrict__ v_out,
                                               float* __restrict__ rref_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int64_t np = C.np;
    // Face nodes are rare; warps without one skip the branch uniformly.
    bool face = false;
    if (C.any_bc) {
        face = on_face(i, j, k, C, false);
        if (face) apply_faces<R, Cd::DEV>(F, i, j, k, n, C, map, vprev);
    }

    // macros (SP:376-388); in deviation form r = rho - 1 and rho = 1 + r
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
    if (face && C.any_pressure && on_face(i, j, k, C, true)) {
        vprev[n] = vx;
        vprev[np + n] = vy;
        vprev[2 * np + n] = vz;
    }
    if constexpr (MACROS) {
        rho_out[n] = rho;
        v_out[n] = vx;
        v_out[np + n] = vy;
        v_out[2 * np + n] = vz;
    }

    collide_sp<R, FORCE, Cd::DEV>(F, r, vx, vy, vz, C);
    store_node<STORE>(F, fout, n, r, rref_out);
}

template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(256, STORE == LBM_STORE_F64 ? 1
                                           : Codec<STORE>::DEV    ? LBM_SP_MINBLOCKS_DEV
                                           : FORCE                ? 4
                                                                  : LBM_SP_MINBLOCKS)
    sp_step_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                                                      const typename Codec<STORE>::T* __restrict__ fin,
                                                      typename Codec<STORE>::T* __restrict__ fout,
                                                      const int32_t* __restrict__ map,
                                                      const uint32_t* __restrict__ coord,
                                                      typename Codec<STORE>::R* __restrict__ vprev,
                                                      typename Codec<STORE>::R* __restrict__ rho_out,
                                                      typename Codec<STORE>::R* __restrict__ v_out,
                                                      const float* __restrict__ rref_in,
                                                      float* __restrict__ rref_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
#if LBM_SP_PDL
    // let the next step's CTAs be scheduled once every CTA of this one runs
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);   // coordinates and map never change between steps
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
#ifdef LBM_DEBUG
    if (i >= C.nx || j >= C.ny || k >= C.nz) {
        lbm_debug_fail(1);
        return;
    }
#endif
#if LBM_SP_PDL
    // populations, node densities and vprev of the previous step: wait for it
    // to complete (returns at once when launched without the attribute)
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif

    R F[19];
    gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k, rref_in);
    sp_finish_node<STORE, FORCE, MACROS>(F, n, i, j, k, C, fout, map, vprev, rho_out, v_out, rref_out);
}

// Initial populations: F = feq(rho, v), then one collision with (rho, v)
// (init SP:160-170 followed by the first step's colission).
template <int STORE, bool FORCE>
__global__ void sp_init_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                               typename Codec<STORE>::T* __restrict__ fout, const float* __restrict__ rho_in,
                               const float* __restrict__ v_in, typename Codec<STORE>::R* __restrict__ vprev,
                               float* __restrict__ rref_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const int64_t np = C.np;
    R rd = (R)0, vx = (R)0, vy = (R)0, vz = (R)0;   // rho - 1 and v
    if (rho_in) {
        rd = (R)rho_in[n] - (R)1;
        vx = (R)v_in[n];
        vy = (R)v_in[np + n];
        vz = (R)v_in[2 * np + n];
    }
    R F[19];
    if constexpr (Cd::DEV) lbm_feq_dev_all<R>(rd, vx, vy, vz, F);
    else lbm_feq_all<R>((R)1 + rd, vx, vy, vz, F);
    vprev[n] = vx;
    vprev[np + n] = vy;
    vprev[2 * np + n] = vz;
    const R r = Cd::DEV ? rd : (R)1 + rd;
    collide_sp<R, FORCE, Cd::DEV>(F, r, vx, vy, vz, C);
    store_node<STORE>(F, fout, n, r, rref_out);
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
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)h->block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = LBM_SP_PDL ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, sp_step_kernel<STORE, FORCE, MACROS>, C, fin, fout,
                                             (const int32_t*)h->d_map, (const uint32_t*)h->d_coord, (R*)h->d_vprev,
                                             (R*)h->d_rho, (R*)h->d_v, (const float*)h->d_rref[h->cur],
                                             h->d_rref[h->cur ^ 1]);
    h->cur ^= 1;
    return lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "sp_step_kernel launch");
}

template <int STORE>
int run_steps(LbmHandle* h, int32_t n, bool macros_last) {
    using R = typename Codec<STORE>::R;
    const SpConsts<R> C = sp_make_consts<R>(h);
#ifdef LBM_DEBUG
    int rc0 = lbm_cuda_check(h, cudaMemcpyToSymbolAsync(g_lbm_debug_nlimit, &h->n_fluid, sizeof(int), 0,
                                                        cudaMemcpyHostToDevice, h->stream),
                             "debug node limit");
    if (!rc0) rc0 = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "debug node limit");
    if (rc0) return rc0;
#endif
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
    float* rref = h->d_rref[h->cur];
    if (h->force) sp_init_kernel<STORE, true><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev, rref);
    else sp_init_kernel<STORE, false><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev, rref);
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
        C.rho_bc_dev[f] = (R)(p.rho_bc[f] - 1.0);
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
    // class (SP:236): /3, /9; scripts (TP:246): 1, 1; standard Guo: 3, 9
    C.gc = p.guo_convention == 0 ? (R)(1.0 / 3.0) : (p.guo_convention == 1 ? (R)1 : (R)3);
    C.gd = p.guo_convention == 0 ? (R)(1.0 / 9.0) : (p.guo_convention == 1 ? (R)1 : (R)9);
    return C;
}
template SpConsts<float> sp_make_consts<float>(const LbmHandle*);
template SpConsts<double> sp_make_consts<double>(const LbmHandle*);

int sp_launch_steps(LbmHandle* h, int32_t n, bool macros_last) {
    if (h->n_fluid == 0) return LBM_OK;   // all solid: nothing to update (an empty grid is not launchable)
    if (h->grey) return grey_launch_steps(h, n, macros_last);
    switch (h->p.storage) {
    case LBM_STORE_F32: return run_steps<LBM_STORE_F32>(h, n, macros_last);
    case LBM_STORE_F16_DEV: return run_steps<LBM_STORE_F16_DEV>(h, n, macros_last);
    case LBM_STORE_BF16_DEV: return run_steps<LBM_STORE_BF16_DEV>(h, n, macros_last);
    case LBM_STORE_F32_DEV: return run_steps<LBM_STORE_F32_DEV>(h, n, macros_last);
    case LBM_STORE_F64: return run_steps<LBM_STORE_F64>(h, n, macros_last);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}

int sp_launch_init(LbmHandle* h, const void* rho_nodes, const void* v_nodes) {
    if (h->n_fluid == 0) return LBM_OK;
    const float* r = (const float*)rho_nodes;
    const float* v = (const float*)v_nodes;
    switch (h->p.storage) {
    case LBM_STORE_F32: return run_init<LBM_STORE_F32>(h, r, v);
    case LBM_STORE_F16_DEV: return run_init<LBM_STORE_F16_DEV>(h, r, v);
    case LBM_STORE_BF16_DEV: return run_init<LBM_STORE_BF16_DEV>(h, r, v);
    case LBM_STORE_F32_DEV: return run_init<LBM_STORE_F32_DEV>(h, r, v);
    case LBM_STORE_F64: return run_init<LBM_STORE_F64>(h, r, v);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}

// Debug builds: the first failed index check since the last call (0 if none),
// cleared on read.  Other builds: always LBM_OK.
int sp_debug_take(LbmHandle* h) {
#ifdef LBM_DEBUG
    int flag = 0;
    const int zero = 0;
    int rc = lbm_cuda_check(h, cudaMemcpyFromSymbol(&flag, g_lbm_debug, sizeof(int)), "debug flag");
    if (!rc && flag) {
        rc = lbm_cuda_check(h, cudaMemcpyToSymbol(g_lbm_debug, &zero, sizeof(int)), "debug flag");
        if (!rc)
            rc = lbm_set_err(h, LBM_EINVAL, flag == 1 ? "debug check: node coordinates outside the lattice"
                                                      : "debug check: neighbour map entry beyond the fluid-node count");
    }
    return rc;
#else
    (void)h;
    return LBM_OK;
#endif
}

int sp_launch_debug_stream(LbmHandle* h, const float* d_in, float* d_out) {
    if (h->n_fluid == 0) return LBM_OK;
    const SpConsts<float> C = sp_make_consts<float>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    sp_gather_kernel<<<grid, h->block, 0, h->stream>>>(C, d_in, d_out, h->d_map, h->d_coord);
    return lbm_cuda_check(h, cudaGetLastError(), "sp_gather_kernel launch");
}
