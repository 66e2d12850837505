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

#include <algorithm>
#include <cstdlib>

#include "lbm_common.cuh"
#include "lbm_internal.h"
#include "lbm_kernels.cuh"

// Resident 256-thread CTAs per SM requested for the step kernel (caps
// registers at 65536 / (256 * n)), as measured on the 256^3 pack (MLUPS):
//  * FP32 reference arithmetic: 6 (40 registers); 4 with the dense Guo forcing;
//  * FP32 deviation form: 6 (40 registers, no spill): 35.3k against 34.9k at 5,
//    forced 37.1k against 36.9k;
//  * 16-bit codecs: 6 (40 registers, 16-24 bytes spilled): FP16 32.2k / BF16
//    32.8k against 32.0k / 32.5k at 4 (64 registers) and 29.5k / 30.2k at 5
//    (48 registers, 68 bytes spilled); forced, 4 is ahead (33.4k / 34.0k
//    against 33.3k / 33.8k at 6).
#ifndef LBM_SP_MINBLOCKS
#define LBM_SP_MINBLOCKS 6
#endif
#ifndef LBM_SP_MINBLOCKS_DEV
#define LBM_SP_MINBLOCKS_DEV 6
#endif
#ifndef LBM_SP_MINBLOCKS_16
#define LBM_SP_MINBLOCKS_16 6
#endif
#ifndef LBM_SP_MINBLOCKS_16F
#define LBM_SP_MINBLOCKS_16F 4
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
                                               typename Codec<STORE>::R* __restrict__ v_out) {
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
    store_node<STORE>(F, fout, n, lbm_ref_at(sp_ref(C), i), C.seed);
}

template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(256, STORE == LBM_STORE_F64 ? 1
                                           : Codec<STORE>::RHOREF ? (FORCE ? LBM_SP_MINBLOCKS_16F : LBM_SP_MINBLOCKS_16)
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
                                                      typename Codec<STORE>::R* __restrict__ v_out) {
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
    gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k, sp_ref(C));
    sp_finish_node<STORE, FORCE, MACROS>(F, n, i, j, k, C, fout, map, vprev, rho_out, v_out);
}

// ------------------------------------------------------------ staged step
// Persistent form of the step over tiles of SPT consecutive nodes (one thread
// per node).  CTAs claim tiles in increasing order from a device counter, so
// uneven tiles and SMs balance out and the tiles in flight stay a compact
// window of the node list (a static tile-to-CTA assignment was 31% slower on
// the 256^3 pack: per-CTA differences add up over its ~25 tiles and the CTAs
// drift apart).  Before a tile is gathered, its packed coordinates -- and,
// when the tile lies in one z plane away from the y faces, the map rows its
// pulls can touch (rows j0 - 1 .. j1 + 1 of planes k - 1, k, k + 1) -- are in
// shared memory, fetched by the bulk-copy (TMA) engine while the CTA worked on
// the tile before, so a node's neighbour lookups are shared-memory reads and
// only its population loads go to HBM.  Other tiles read the map from global
// memory as sp_step_kernel does.
//
// Protocol (per staging buffer: one mbarrier, a release counter, the tile
// index): the last warp to finish gathering the buffer's tile claims the next
// tile and issues its copies (or, when no tile is left, arrives on the
// mbarrier without copies and stores -1); the copies land while the CTA
// collides and stores.  The counter is never reset: launch e claims values
// base_e, base_e + 1, ... after griddepcontrol.wait (so consecutive launches
// never interleave their claims), each buffer of each CTA ends with exactly one
// failed claim, and a launch therefore consumes ntile + SPT_STAGES * G values,
// by which the host advances base.  Waits on the mbarriers are bounded (~1 s);
// on a timeout the CTA records g_sp_stage_err, waits once more (bounded) for
// its own copies and leaves.
constexpr int SPT = 256;            // nodes per tile = threads per CTA
constexpr int SPT_WARPS = SPT / 32;
// Staging buffers per CTA: 1 = the next tile's copies are issued when every
// warp has gathered the current one; 2 = one tile further ahead.
#ifndef LBM_SPT_STAGES
#define LBM_SPT_STAGES 1
#endif
constexpr int SPT_STAGES = LBM_SPT_STAGES;
// Diagnostics (tuning builds): 1 = gather through the global map even when the tile is staged.
#ifndef LBM_SPT_GLOBALMAP
#define LBM_SPT_GLOBALMAP 0
#endif
#ifndef LBM_SPT_SMEM
#define LBM_SPT_SMEM (24 * 1024)
#endif
constexpr int SPT_SMEM = LBM_SPT_SMEM;  // shared-memory budget of one staging buffer
constexpr int SPT_BY_MAX = 32;      // staged rows per plane at most
constexpr int SPT_HDR = 32;         // mbarriers, release counters, tile indices
constexpr long long SPT_WAIT_CYCLES = 2000000000LL;

struct SptArgs {
    const int2* tinfo;              // per tile: {first staged row, k | rows << 16} (rows 0: not staged)
    unsigned long long* ctr;        // tile claims (never reset)
    unsigned long long base;        // counter value at this launch's first claim
    int32_t ntile;
    int32_t plane;                  // ints per staged plane (16-byte multiple)
    int32_t np;
};

// Rows a staged plane holds: as many whole x rows as fit the budget (3 planes), at most SPT_BY_MAX.
__host__ __device__ inline int spt_rows_max(int nx) {
    const int r = (SPT_SMEM - SPT_HDR - SPT * 4 - 3 * 12 * 4) / (3 * 4 * nx);
    return r < SPT_BY_MAX ? r : SPT_BY_MAX;
}
// ints per staged plane: the rows, the alignment shift (< 4) and the rounding
// of the copy to 16 bytes (< 4), as a multiple of 4 ints
__host__ __device__ inline int spt_plane_ints(int nx) { return (spt_rows_max(nx) * nx + 8 + 3) / 4 * 4; }

__device__ int g_sp_stage_err;

__device__ __forceinline__ uint32_t spt_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool spt_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(spt_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > SPT_WAIT_CYCLES) return false;
    }
}

__device__ __forceinline__ void spt_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(spt_u32(dst)), "l"(src), "r"(bytes), "r"(spt_u32(bar))
                 : "memory");
}

// Plane pz of a staged tile: first map element (16-byte aligned) and the
// shift of the first staged row's cell 0 from it.
__device__ __forceinline__ void spt_plane(int pz, int k, int row0, int nx, int ny, int nz, int64_t* first, int* shift) {
    int kz = k - 1 + pz;
    kz = kz < 0 ? kz + nz : (kz >= nz ? kz - nz : kz);
    const int64_t off = ((int64_t)kz * ny + row0) * nx;
    *first = off & ~(int64_t)3;
    *shift = (int)(off - *first);
}

// Claim the next tile for one staging buffer and issue its copies, or, when
// no tile is left, store -1 and complete the buffer's phase without copies
// (one thread).
__device__ __forceinline__ void spt_next(const SptArgs& A, int nx, int ny, int nz, const uint32_t* coord,
                                         const int32_t* map, uint64_t* bar, int* s_tile, uint32_t* s_coord,
                                         int32_t* s_map) {
    const unsigned long long v = atomicAdd(A.ctr, 1ull) - A.base;
    if (v >= (unsigned long long)A.ntile) {
        *s_tile = -1;
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(spt_u32(bar)) : "memory");
        return;
    }
    const int t = (int)v;
    *s_tile = t;
    const int2 ti = A.tinfo[t];
    const int base = t * SPT;
    const uint32_t cbytes = (uint32_t)min(SPT, A.np - base) * 4u;   // np is a multiple of 64
    const int rows = (ti.y >> 16) & 0xff, k = ti.y & 0xffff;
    uint32_t pbytes[3] = {0, 0, 0};
    int64_t first[3] = {0, 0, 0};
    if (rows) {
        for (int pz = 0; pz < 3; ++pz) {
            int sh;
            spt_plane(pz, k, ti.x, nx, ny, nz, &first[pz], &sh);
            pbytes[pz] = (uint32_t)(((rows * nx + sh) * 4 + 15) & ~15);
        }
    }
    const uint32_t tx = cbytes + pbytes[0] + pbytes[1] + pbytes[2];
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(spt_u32(bar)), "r"(tx) : "memory");
    spt_bulk(s_coord, coord + base, cbytes, bar);
    if (rows)
        for (int pz = 0; pz < 3; ++pz) spt_bulk(s_map + pz * A.plane, map + first[pz], pbytes[pz], bar);
}

template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(SPT, STORE == LBM_STORE_F64 ? 1
                                       : Codec<STORE>::RHOREF ? (FORCE ? LBM_SP_MINBLOCKS_16F : LBM_SP_MINBLOCKS_16)
                                       : Codec<STORE>::DEV    ? LBM_SP_MINBLOCKS_DEV
                                       : FORCE                ? 4
                                                              : LBM_SP_MINBLOCKS)
    sp_tile_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C, const __grid_constant__ SptArgs A,
                   const typename Codec<STORE>::T* __restrict__ fin, typename Codec<STORE>::T* __restrict__ fout,
                   const int32_t* __restrict__ map, const uint32_t* __restrict__ coord,
                   typename Codec<STORE>::R* __restrict__ vprev, typename Codec<STORE>::R* __restrict__ rho_out,
                   typename Codec<STORE>::R* __restrict__ v_out) {
    using R = typename Codec<STORE>::R;
    extern __shared__ __align__(16) unsigned char spt_smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(spt_smem);
    int* rels = reinterpret_cast<int*>(spt_smem + 16);
    int* tiles = reinterpret_cast<int*>(spt_smem + 24);
    const int stage_bytes = SPT * 4 + 3 * A.plane * 4;
#if LBM_SP_PDL
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
    if (threadIdx.x == 0) {
        for (int q = 0; q < SPT_STAGES; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(spt_u32(bars + q)), "r"(1) : "memory");
            rels[q] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
#if LBM_SP_PDL
    // the previous step complete: its claims are all made, its populations written
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
    if (threadIdx.x == 0)
        for (int q = 0; q < SPT_STAGES; ++q) {
            unsigned char* sb = spt_smem + SPT_HDR + q * stage_bytes;
            spt_next(A, C.nx, C.ny, C.nz, coord, map, bars + q, tiles + q, reinterpret_cast<uint32_t*>(sb),
                     reinterpret_cast<int32_t*>(sb + SPT * 4));
        }
    const int lane = threadIdx.x & 31;
    for (uint32_t it = 0;; ++it) {
        const int q = SPT_STAGES == 1 ? 0 : (int)(it % SPT_STAGES);
        const uint32_t parity = (it / SPT_STAGES) & 1;
        uint64_t* bar = bars + q;
        unsigned char* sb = spt_smem + SPT_HDR + q * stage_bytes;
        uint32_t* s_coord = reinterpret_cast<uint32_t*>(sb);
        int32_t* s_map = reinterpret_cast<int32_t*>(sb + SPT * 4);
        if (!spt_wait(bar, parity)) {
            if (threadIdx.x == 0) atomicExch(&g_sp_stage_err, 1);
            spt_wait(bar, parity);
            return;
        }
        const int t = tiles[q];
        if (t < 0) break;                       // no tile left (no copies in flight: claims only fail from here on)
        const int n = t * SPT + threadIdx.x;
        const bool active = n < C.n_fluid;
        const uint32_t pc = s_coord[threadIdx.x];
        const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
        R F[19];
        if (active) {
#ifdef LBM_DEBUG
            if (i >= C.nx || j >= C.ny || k >= C.nz) lbm_debug_fail(1);
#endif
            const int2 ti = A.tinfo[t];
            const int rows = (ti.y >> 16) & 0xff;
            if (rows && !LBM_SPT_GLOBALMAP) {
                int b[3];
#pragma unroll
                for (int pz = 0; pz < 3; ++pz) {
                    int64_t first;
                    int sh;
                    spt_plane(pz, k, ti.x, C.nx, C.ny, C.nz, &first, &sh);
                    b[pz] = pz * A.plane + sh + (j - ti.x) * C.nx + i;
                }
                gather_node_smem<STORE>(F, fin, s_map, b, n, C.nx, i, sp_ref(C));
            } else {
                gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k, sp_ref(C));
            }
        }
        // this warp is done with the buffer; the last warp claims and stages the next tile
        __syncwarp();
        __threadfence_block();
        if (lane == 0 && atomicAdd(rels + q, 1) == SPT_WARPS - 1) {
            __threadfence_block();
            atomicExch(rels + q, 0);
            // the buffer is overwritten by the async proxy after these generic reads
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            spt_next(A, C.nx, C.ny, C.nz, coord, map, bar, tiles + q, s_coord, s_map);
        }
        if (active) sp_finish_node<STORE, FORCE, MACROS>(F, n, i, j, k, C, fout, map, vprev, rho_out, v_out);
    }
}

// One-tile form of the staged step: CTA b advances tile b (no persistent
// loop).  Thread 0 copies the tile's coordinates and map rows into shared
// memory with the bulk-copy engine; coordinates and map never change, so the
// copies are made before griddepcontrol.wait and overlap the previous step's
// drain for the CTAs resident by then.
template <int STORE, bool FORCE, bool MACROS>
__global__ void __launch_bounds__(SPT, STORE == LBM_STORE_F64 ? 1
                                       : Codec<STORE>::RHOREF ? (FORCE ? LBM_SP_MINBLOCKS_16F : LBM_SP_MINBLOCKS_16)
                                       : Codec<STORE>::DEV    ? LBM_SP_MINBLOCKS_DEV
                                       : FORCE                ? 4
                                                              : LBM_SP_MINBLOCKS)
    sp_tile1_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C, const __grid_constant__ SptArgs A,
                    const typename Codec<STORE>::T* __restrict__ fin, typename Codec<STORE>::T* __restrict__ fout,
                    const int32_t* __restrict__ map, const uint32_t* __restrict__ coord,
                    typename Codec<STORE>::R* __restrict__ vprev, typename Codec<STORE>::R* __restrict__ rho_out,
                    typename Codec<STORE>::R* __restrict__ v_out) {
    using R = typename Codec<STORE>::R;
    extern __shared__ __align__(16) unsigned char spt_smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(spt_smem);
    uint32_t* s_coord = reinterpret_cast<uint32_t*>(spt_smem + SPT_HDR);
    int32_t* s_map = reinterpret_cast<int32_t*>(spt_smem + SPT_HDR + SPT * 4);
#if LBM_SP_PDL
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
    const int t = blockIdx.x;
    const int2 ti = A.tinfo[t];
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(spt_u32(bar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const int base = t * SPT;
        const uint32_t cbytes = (uint32_t)min(SPT, A.np - base) * 4u;   // np is a multiple of 64
        const int rows = (ti.y >> 16) & 0xff, k = ti.y & 0xffff;
        uint32_t pbytes[3] = {0, 0, 0};
        int64_t first[3] = {0, 0, 0};
        if (rows && !LBM_SPT_GLOBALMAP) {
            for (int pz = 0; pz < 3; ++pz) {
                int sh;
                spt_plane(pz, k, ti.x, C.nx, C.ny, C.nz, &first[pz], &sh);
                pbytes[pz] = (uint32_t)(((rows * C.nx + sh) * 4 + 15) & ~15);
            }
        }
        const uint32_t tx = cbytes + pbytes[0] + pbytes[1] + pbytes[2];
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(spt_u32(bar)), "r"(tx) : "memory");
        spt_bulk(s_coord, coord + base, cbytes, bar);
        for (int pz = 0; pz < 3; ++pz)
            if (pbytes[pz]) spt_bulk(s_map + pz * A.plane, map + first[pz], pbytes[pz], bar);
    }
    __syncthreads();   // the mbarrier is initialised before anyone waits on it
    if (!spt_wait(bar, 0)) {
        if (threadIdx.x == 0) atomicExch(&g_sp_stage_err, 1);
        spt_wait(bar, 0);
        return;
    }
    const int n = t * SPT + threadIdx.x;
    if (n >= C.n_fluid) return;
    const uint32_t pc = s_coord[threadIdx.x];
    const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
#ifdef LBM_DEBUG
    if (i >= C.nx || j >= C.ny || k >= C.nz) {
        lbm_debug_fail(1);
        return;
    }
#endif
    const int rows = (ti.y >> 16) & 0xff;
    int b[3];
    if (rows && !LBM_SPT_GLOBALMAP) {
#pragma unroll
        for (int pz = 0; pz < 3; ++pz) {
            int64_t first;
            int sh;
            spt_plane(pz, k, ti.x, C.nx, C.ny, C.nz, &first, &sh);
            b[pz] = pz * A.plane + sh + (j - ti.x) * C.nx + i;
        }
    }
#if LBM_SP_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
    R F[19];
    if (rows && !LBM_SPT_GLOBALMAP) gather_node_smem<STORE>(F, fin, s_map, b, n, C.nx, i, sp_ref(C));
    else gather_node<STORE>(F, fin, map, n, C.nx, C.ny, C.nz, i, j, k, sp_ref(C));
    sp_finish_node<STORE, FORCE, MACROS>(F, n, i, j, k, C, fout, map, vprev, rho_out, v_out);
}

size_t spt1_smem_bytes(int nx) { return SPT_HDR + SPT * 4 + 3 * (size_t)spt_plane_ints(nx) * 4; }

// Per tile of the staged step: the first staged row and the plane, or rows = 0
// when the tile is not staged (it spans two z planes, touches a y face, or
// covers more rows than a staged plane holds).
__global__ void spt_info_kernel(const uint32_t* __restrict__ coord, int n_fluid, int ntile, int ny, int rows_max,
                                int2* __restrict__ tinfo) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntile) return;
    const int first = t * SPT, last = min(first + SPT, n_fluid) - 1;
    const uint32_t a = coord[first], b = coord[last];
    const int k0 = lbm_pk(a), k1 = lbm_pk(b), j0 = lbm_pj(a), j1 = lbm_pj(b);
    const int rows = j1 - j0 + 3;
    const bool staged = k0 == k1 && j0 >= 1 && j1 <= ny - 2 && rows <= rows_max;
    tinfo[t] = make_int2(j0 - 1, k0 | ((staged ? rows : 0) << 16));
}

size_t spt_smem_bytes(int nx) { return SPT_HDR + SPT_STAGES * (SPT * 4 + 3 * (size_t)spt_plane_ints(nx) * 4); }

// Initial populations: F = feq(rho, v), then one collision with (rho, v)
// (init SP:160-170 followed by the first step's colission).
template <int STORE, bool FORCE>
__global__ void sp_init_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                               typename Codec<STORE>::T* __restrict__ fout, const float* __restrict__ rho_in,
                               const float* __restrict__ v_in, typename Codec<STORE>::R* __restrict__ vprev,
                               const uint32_t* __restrict__ coord) {
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
    store_node<STORE>(F, fout, n, lbm_ref_at(sp_ref(C), lbm_pi(coord[n])), ~C.seed);
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
                                             (R*)h->d_rho, (R*)h->d_v);
    h->cur ^= 1;
    return lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "sp_step_kernel launch");
}

template <int STORE, bool FORCE, bool MACROS>
int launch_tile(LbmHandle* h, const SpConsts<typename Codec<STORE>::R>& C, const SptArgs& A, int grid, size_t smem) {
    using T = typename Codec<STORE>::T;
    using R = typename Codec<STORE>::R;
    const T* fin = (const T*)h->d_f[h->cur];
    T* fout = (T*)h->d_f[h->cur ^ 1];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(SPT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = LBM_SP_PDL ? 1 : 0;
    SptArgs a = A;
    a.base = h->spt_base;
    if (h->tiled_mode == 2) {
        cfg.gridDim = dim3((unsigned)A.ntile);
        cfg.dynamicSmemBytes = spt1_smem_bytes(h->p.nx);
        const cudaError_t e1 = cudaLaunchKernelEx(&cfg, sp_tile1_kernel<STORE, FORCE, MACROS>, C, a, fin, fout,
                                                  (const int32_t*)h->d_map, (const uint32_t*)h->d_coord,
                                                  (R*)h->d_vprev, (R*)h->d_rho, (R*)h->d_v);
        const int rc1 = lbm_cuda_check(h, e1 != cudaSuccess ? e1 : cudaGetLastError(), "sp_tile1_kernel launch");
        if (!rc1) h->cur ^= 1;
        return rc1;
    }
    const cudaError_t e = cudaLaunchKernelEx(&cfg, sp_tile_kernel<STORE, FORCE, MACROS>, C, a, fin, fout,
                                             (const int32_t*)h->d_map, (const uint32_t*)h->d_coord, (R*)h->d_vprev,
                                             (R*)h->d_rho, (R*)h->d_v);
    const int rc = lbm_cuda_check(h, e != cudaSuccess ? e : cudaGetLastError(), "sp_tile_kernel launch");
    if (!rc) {
        h->cur ^= 1;
        h->spt_base += (unsigned long long)A.ntile + (unsigned long long)SPT_STAGES * grid;
    }
    return rc;
}

// Resident CTAs of the staged kernel on the whole device (its persistent grid).
template <int STORE, bool FORCE>
int tile_grid(LbmHandle* h, size_t smem) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sp_tile_kernel<STORE, FORCE, false>, SPT, smem) !=
            cudaSuccess ||
        occ < 1)
        occ = 1;
    return (int)std::min<int64_t>((int64_t)occ * h->sm_count, h->ntile);
}

template <int STORE>
int run_tiles(LbmHandle* h, int32_t n, bool macros_last) {
    using R = typename Codec<STORE>::R;
    SpConsts<R> C = sp_make_consts<R>(h);
    const size_t smem = spt_smem_bytes(h->p.nx);
    SptArgs A;
    A.tinfo = h->d_tinfo;
    A.ctr = h->d_spt_ctr;
    A.base = 0;
    A.ntile = h->ntile;
    A.plane = spt_plane_ints(h->p.nx);
    A.np = (int32_t)h->np;
    const int grid = h->force ? tile_grid<STORE, true>(h, smem) : tile_grid<STORE, false>(h, smem);
    for (int32_t it = 0; it < n; ++it) {
        const bool mac = macros_last && it == n - 1;
        C.seed = (uint32_t)(h->steps_done + it);   // global step index: rounding bits of this step
        int rc;
        if (h->force) rc = mac ? launch_tile<STORE, true, true>(h, C, A, grid, smem) : launch_tile<STORE, true, false>(h, C, A, grid, smem);
        else rc = mac ? launch_tile<STORE, false, true>(h, C, A, grid, smem) : launch_tile<STORE, false, false>(h, C, A, grid, smem);
        if (rc) return rc;
    }
    return LBM_OK;
}

template <int STORE>
int run_steps(LbmHandle* h, int32_t n, bool macros_last) {
    using R = typename Codec<STORE>::R;
    SpConsts<R> C = sp_make_consts<R>(h);
#ifdef LBM_DEBUG
    int rc0 = lbm_cuda_check(h, cudaMemcpyToSymbolAsync(g_lbm_debug_nlimit, &h->n_fluid, sizeof(int), 0,
                                                        cudaMemcpyHostToDevice, h->stream),
                             "debug node limit");
    if (!rc0) rc0 = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "debug node limit");
    if (rc0) return rc0;
#endif
    if (h->tiled) return run_tiles<STORE>(h, n, macros_last);
    const int grid = (int)((h->n_fluid + h->block - 1) / h->block);
    for (int32_t it = 0; it < n; ++it) {
        const bool mac = macros_last && it == n - 1;
        C.seed = (uint32_t)(h->steps_done + it);   // global step index: rounding bits of this step
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
    const uint32_t* coord = h->d_coord;
    if (h->force) sp_init_kernel<STORE, true><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev, coord);
    else sp_init_kernel<STORE, false><<<grid, h->block, 0, h->stream>>>(C, fout, rho, v, (R*)h->d_vprev, coord);
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
    // reference density of the 16-bit codecs: the linear profile between the
    // two x faces when both hold a fixed pressure, else 0
    C.ref_a = (R)0;
    C.ref_b = (R)0;
    if (p.bc[0] == LBM_BC_PRESSURE && p.bc[1] == LBM_BC_PRESSURE && p.nx > 1) {
        C.ref_a = (R)(p.rho_bc[0] - 1.0);
        C.ref_b = (R)((p.rho_bc[1] - p.rho_bc[0]) / (double)(p.nx - 1));
    }
    C.seed = (uint32_t)h->steps_done;
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

// Per-tile staging plan of the staged step kernels (after the index is built),
// chosen by LBM_SP_TILED in the environment: 0 or unset = sp_step_kernel (the
// default: fastest measured), 1 = persistent staged kernel, 2 = one staged tile
// per CTA.  256^3 pack, FP32 / f32dev / FP16 MLUPS on one GB300: sp_step_kernel
// 34.6k / 35.4k / 31.8k; persistent staged 29.2k / 29.9k / 29.4k; one tile per
// CTA 28.6k / 28.9k / 28.4k, and 32.3k / 32.9k / 29.1k when that kernel stages
// only the coordinates and reads the map from global memory: the L1 already
// serves the map lookups, so staging the rows adds a copy before the gather
// and takes L1 capacity without shortening the coordinates -> populations chain.
int sp_tiles_setup(LbmHandle* h) {
    if (h->d_tinfo) cudaFree(h->d_tinfo);
    h->d_tinfo = nullptr;
    h->d_spt_ctr = nullptr;
    h->spt_base = 0;
    h->ntile = 0;
    h->tiled = false;
    const char* env = getenv("LBM_SP_TILED");
    h->tiled_mode = env ? atoi(env) : 0;
    if (h->tiled_mode == 0 || h->n_fluid == 0 || spt_rows_max(h->p.nx) < 3) return LBM_OK;
    h->ntile = (int32_t)((h->n_fluid + SPT - 1) / SPT);
    // tile plan and, behind it, the 8-byte claim counter
    const size_t tbytes = (sizeof(int2) * h->ntile + 15) / 16 * 16;
    int rc = lbm_cuda_check(h, cudaMalloc((void**)&h->d_tinfo, tbytes + 16), "tile plan");
    if (rc) return rc;
    h->device_bytes += tbytes + 16;
    h->d_spt_ctr = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(h->d_tinfo) + tbytes);
    rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_spt_ctr, 0, 8, h->stream), "tile claim counter");
    if (rc) return rc;
    spt_info_kernel<<<(h->ntile + 255) / 256, 256, 0, h->stream>>>(h->d_coord, h->n_fluid, h->ntile, h->p.ny,
                                                                  spt_rows_max(h->p.nx), h->d_tinfo);
    rc = lbm_cuda_check(h, cudaGetLastError(), "spt_info_kernel launch");
    if (!rc) h->tiled = true;
    return rc;
}

// Failed checks of the last steps, cleared on read: a staged-step copy that
// timed out (any build) and, in -DLBM_DEBUG builds, the first failed index
// check.  LBM_OK when nothing failed.
int sp_debug_take(LbmHandle* h) {
    if (h->tiled) {
        int err = 0;
        const int zero = 0;
        int rc = lbm_cuda_check(h, cudaMemcpyFromSymbol(&err, g_sp_stage_err, sizeof(int)), "staging flag");
        if (!rc && err) {
            rc = lbm_cuda_check(h, cudaMemcpyToSymbol(g_sp_stage_err, &zero, sizeof(int)), "staging flag");
            // an abandoned launch left its claims unfinished: restart the counter
            if (!rc) rc = lbm_cuda_check(h, cudaMemset(h->d_spt_ctr, 0, 8), "tile claim counter");
            h->spt_base = 0;
            if (!rc) rc = lbm_set_err(h, LBM_ECUDA, "step kernel: a shared-memory staging copy did not complete in time");
        }
        if (rc) return rc;
    }
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
