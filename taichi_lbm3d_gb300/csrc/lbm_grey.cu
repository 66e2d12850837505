// Grey-scale (partial bounce-back) single-phase step over the compacted
// fluid-node list.  GS = Grey_Scale/lbm_solver_3d_Macro_Sukop.py (taichi_LBM3D tree).
//
// The reference's sweeps per step (GS:330-336) are colission (GS:203-218),
// streaming0 (GS:234-240), streaming1 (GS:243-252), Boundary_condition on the
// x faces (GS:263-293) and streaming3 (GS:296-312).  In pull form, with the
// post-collision populations f as the state between launches, a fluid node x
// receives for each direction s from y = x - e_s (periodic wrap):
//   y fluid:  F[s] = f(y)[s] + ns(y) (f(x)[LR s] - f(y)[s])
//             (streaming0 at y mixes with the opposite population of the
//             cell the population moves to, which is x itself)
//   y solid:  F[s] keeps its previous value: streaming1 only pushes from
//             fluid cells, so that slot still holds init's feq(s, 1, 0) = w_s,
//             or, on a fixed-velocity x face, what the face rule wrote last step
// then the x faces, rho/v (+ F/2 rho), and the single-phase MRT collision with
// the script's Guo term (same arithmetic as the single-phase step).
//
// Extra per-node data: ns (grey value) [np].  Fixed-velocity x faces keep
// their post-face F in a side array [2][ny*nz][19] (the in-place face rule
// reads the stale slots), initialised to w_s by lbm_init.
#include <cuda_runtime.h>

#include "lbm_common.cuh"
#include "lbm_internal.h"
#include "lbm_kernels.cuh"

namespace {
using namespace lbmk;

// Value of a slot that no fluid cell pushes into: feq(s, 1, 0) = w_s (GS:120-127);
// 0 in deviation form.
template <int S, typename R, bool DEV>
__device__ __forceinline__ R grey_rest() {
    return DEV ? (R)0 : (R)lbm_w(S);
}

template <int STORE, bool XWRAP>
struct GreyGather {
    using Cd = Codec<STORE>;
    using T = typename Cd::T;
    using R = typename Cd::R;
    using NS = R;
    template <int S>
    static __device__ __forceinline__ void one(R* F, const R* Fo, const T* __restrict__ fin,
                                               const int32_t* __restrict__ map, const NS* __restrict__ ns,
                                               const Rows& rows, int i, int xm, int xp, const RefX<R>& rx) {
        const int src = pull_source<S, XWRAP>(map, rows, i, xm, xp);
        if (src >= 0) {
            R a = Cd::template dec<S>(fin[lbm_eoff32(src) + 32 * S]);
            if constexpr (Cd::RHOREF) {
                R rs = rx.ri;
                if constexpr (lbm_ex(S) != 0) {
                    const int xs = lbm_ex(S) > 0 ? xm : xp;
                    if constexpr (XWRAP) rs = lbm_fma<R>(rx.b, (R)xs, rx.a);
                    else rs = lbm_ex(S) > 0 ? rx.ri - rx.b : rx.ri + rx.b;
                }
                a = lbm_fma<R>((R)lbm_w(S), rs, a);
            }
            F[S] = a + __ldg(ns + src) * (Fo[lbm_lr(S)] - a);
        } else {
            F[S] = grey_rest<S, R, Cd::DEV>();
        }
    }
};

template <int STORE>
__device__ __forceinline__ void grey_gather_node(typename Codec<STORE>::R* F, const typename Codec<STORE>::T* __restrict__ fin,
                                                 const int32_t* __restrict__ map,
                                                 const typename Codec<STORE>::R* __restrict__ ns, int n, int nx, int ny,
                                                 int nz, int i, int j, int k,
                                                 const LbmRef<typename Codec<STORE>::R>& ref) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int xm = i == 0 ? nx - 1 : i - 1, xp = i == nx - 1 ? 0 : i + 1;
    const int ym = j == 0 ? ny - 1 : j - 1, yp = j == ny - 1 ? 0 : j + 1;
    const int zm = k == 0 ? nz - 1 : k - 1, zp = k == nz - 1 ? 0 : k + 1;
    const Rows rows = make_rows(nx, ny, i, j, k, ym, yp, zm, zp);
    // the node's own post-collision populations (the partners of the mixing)
    const typename Cd::T* own = fin + lbm_eoff32(n);
    const auto rx = ref_x<STORE>(ref, i);
    R Fo[19];
#define LBM_OWN(S)                                                                        \
    Fo[S] = Cd::template dec<S>(own[32 * S]);                                             \
    if constexpr (Cd::RHOREF) Fo[S] = lbm_fma<R>((R)lbm_w(S), rx.ri, Fo[S]);
    LBM_OWN(0) LBM_ALL_DIRS(LBM_OWN)
#undef LBM_OWN
    F[0] = Fo[0] + ns[n] * (Fo[0] - Fo[0]);
    const bool x_inside = i > 0 && i < nx - 1;
    if (__all_sync(__activemask(), x_inside)) {
#define LBM_G(S) GreyGather<STORE, false>::template one<S>(F, Fo, fin, map, ns, rows, i, xm, xp, rx);
        LBM_ALL_DIRS(LBM_G)
#undef LBM_G
    } else {
#define LBM_G(S) GreyGather<STORE, true>::template one<S>(F, Fo, fin, map, ns, rows, i, xm, xp, rx);
        LBM_ALL_DIRS(LBM_G)
#undef LBM_G
    }
}

// Fixed-velocity x face: slots whose upstream cell is solid hold what the face
// rule wrote at the previous step (side array), not w_s.
template <typename R>
__device__ __forceinline__ void grey_face_restore(R* F, int i, int j, int k, const SpConsts<R>& C,
                                                  const int32_t* __restrict__ map, const R* st) {
    const int xm = i == 0 ? C.nx - 1 : i - 1, xp = i == C.nx - 1 ? 0 : i + 1;
    const int ym = j == 0 ? C.ny - 1 : j - 1, yp = j == C.ny - 1 ? 0 : j + 1;
    const int zm = k == 0 ? C.nz - 1 : k - 1, zp = k == C.nz - 1 ? 0 : k + 1;
    const Rows rows = make_rows(C.nx, C.ny, i, j, k, ym, yp, zm, zp);
#define LBM_R(S) \
    if (pull_source<S, true>(map, rows, i, xm, xp) < 0) F[S] = st[S];
    LBM_ALL_DIRS(LBM_R)
#undef LBM_R
}

// 4 CTAs of 256 per SM (64 registers); the density-referenced 16-bit codecs,
// which gather the source densities as well, 3 (80 registers): on the 256^3
// grey field FP16 runs 25.7k MLUPS at 3 against 24.4k at 4, while FP32 and
// f32dev lose 6% and 11% at 3.
template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(256, STORE == LBM_STORE_F64 ? 1 : (Codec<STORE>::RHOREF ? 3 : 4)) grey_step_kernel(
    const __grid_constant__ SpConsts<typename Codec<STORE>::R> C, const typename Codec<STORE>::T* __restrict__ fin,
    typename Codec<STORE>::T* __restrict__ fout, const int32_t* __restrict__ map, const uint32_t* __restrict__ coord,
    const typename Codec<STORE>::R* __restrict__ ns, typename Codec<STORE>::R* __restrict__ face_stale,
    typename Codec<STORE>::R* __restrict__ vprev, typename Codec<STORE>::R* __restrict__ rho_out,
    typename Codec<STORE>::R* __restrict__ v_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    // programmatic dependent launch, as in the single-phase step: the next
    // step's CTAs may start once all of these run; they wait below before
    // reading populations, grey values' partners or the face side array
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = __ldg(coord + n);
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
    const int64_t np = C.np;
    asm volatile("griddepcontrol.wait;" ::: "memory");

    R F[19];
    grey_gather_node<STORE>(F, fin, map, ns, n, C.nx, C.ny, C.nz, i, j, k, sp_ref(C));

    bool face = false;
    if (C.any_bc) {
        face = on_face(i, j, k, C, false);
        if (face) {
            // x faces only (GS:263-293); velocity faces read and keep their stale slots
            R* st = nullptr;
            if (face_stale && i == 0 && C.bc[0] == LBM_BC_VELOCITY) st = face_stale + (int64_t)19 * (j + C.ny * k);
            if (face_stale && i == C.nx - 1 && C.bc[1] == LBM_BC_VELOCITY)
                st = face_stale + (int64_t)19 * ((int64_t)C.ny * C.nz + j + C.ny * k);
            if (st) grey_face_restore<R>(F, i, j, k, C, map, st);
            apply_faces<R, Cd::DEV>(F, i, j, k, n, C, map, vprev);
            if (st) {
#pragma unroll
                for (int s = 0; s < 19; ++s) st[s] = F[s];
            }
        }
    }

    // streaming3 (GS:296-312)
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
    // colission (GS:203-218): the single-phase MRT collision with the script's Guo term
    collide_sp<R, FORCE, Cd::DEV>(F, r, vx, vy, vz, C);
    store_node<STORE>(F, fout, n, lbm_ref_at(sp_ref(C), i), C.seed);
}

template <int STORE, bool FORCE, bool MACROS>
int launch_grey(LbmHandle* h, const SpConsts<typename Codec<STORE>::R>& C, int grid) {
    using T = typename Codec<STORE>::T;
    using R = typename Codec<STORE>::R;
    const T* fin = (const T*)h->d_f[h->cur];
    T* fout = (T*)h->d_f[h->cur ^ 1];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)h->block);
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, grey_step_kernel<STORE, FORCE, MACROS>, C, fin, fout,
                                             (const int32_t*)h->d_map, (const uint32_t*)h->d_coord,
                                             (const R*)h->d_ns, (R*)h->d_gstale, (R*)h->d_vprev, (R*)h->d_rho,
                                             (R*)h->d_v);
    h->cur ^= 1;
    return lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "grey_step_kernel launch");
}

template <int STORE>
int run_grey(LbmHandle* h, int32_t n, bool macros_last) {
    using R = typename Codec<STORE>::R;
    SpConsts<R> C = sp_make_consts<R>(h);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    for (int32_t it = 0; it < n; ++it) {
        const bool mac = macros_last && it == n - 1;
        C.seed = (uint32_t)(h->steps_done + it);
        int rc;
        if (h->force) rc = mac ? launch_grey<STORE, true, true>(h, C, grid) : launch_grey<STORE, true, false>(h, C, grid);
        else rc = mac ? launch_grey<STORE, false, true>(h, C, grid) : launch_grey<STORE, false, false>(h, C, grid);
        if (rc) return rc;
    }
    return LBM_OK;
}

}  // namespace

int grey_launch_steps(LbmHandle* h, int32_t n, bool macros_last) {
    switch (h->p.storage) {
    case LBM_STORE_F32: return run_grey<LBM_STORE_F32>(h, n, macros_last);
    case LBM_STORE_F16_DEV: return run_grey<LBM_STORE_F16_DEV>(h, n, macros_last);
    case LBM_STORE_BF16_DEV: return run_grey<LBM_STORE_BF16_DEV>(h, n, macros_last);
    case LBM_STORE_F32_DEV: return run_grey<LBM_STORE_F32_DEV>(h, n, macros_last);
    case LBM_STORE_F64: return run_grey<LBM_STORE_F64>(h, n, macros_last);
    }
    return lbm_set_err(h, LBM_EINVAL, "unknown storage");
}
