// K5: many independent porous subvolumes advanced by one persistent kernel per
// time step, `check_every` steps captured into one CUDA graph.
//
// Layout: the compacted fluid nodes of all subvolumes are concatenated (each
// subvolume starts on a multiple of 32 so no population chunk straddles two);
// each subvolume has its own dense node map holding node indices local to the
// subvolume.  A CTA offsets the population, coordinate and density-reference
// arrays to its subvolume's first node once (64-bit), and the 32-bit offset
// arithmetic of the gather stays local, so the batch as a whole may exceed
// 2^31 population elements.  Work is cut into tiles (subvolume, local node
// range); the grid is sized to the resident CTAs of
// the GPU and CTAs claim tiles from an atomic counter, so uneven subvolumes
// share the GPU without tail effects.  Converged subvolumes are removed by
// rewriting the tile list in device memory between graph launches; the graph
// itself never changes.  The node update is the single-phase step of K1 (all
// faces periodic, optional body force) in any storage mode.
//
// Convergence: the last step of each graph writes, per tile, the FP64 sum of
// v along x; the host sums tiles in order per subvolume (deterministic) and
// compares the Darcy velocity with the previous check.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "lbm_kernels.cuh"

struct BatchSub {
    int32_t nx, ny, nz, n_fluid;
    int64_t map_off;        // first cell of this subvolume's dense map
    int64_t node_begin;     // first node (a multiple of 32) in the concatenated arrays
};

struct BatchTile {
    int32_t sub, begin, end, pad;   // local node range [begin, end)
};

// Per-subvolume views of the concatenated arrays (node indices become local).
template <typename T>
__device__ __forceinline__ T* sub_pop(T* f, int64_t node_begin) {
    return f + lbm_eoff(node_begin);
}
template <typename T>
__device__ __forceinline__ T* sub_node(T* a, int64_t node_begin) {
    return a ? a + node_begin : a;
}

struct LbmBatch {
    LbmHandle h;                        // shared params, stream, populations, coords, map
    std::vector<BatchSub> subs;
    std::vector<int32_t> tile_len;      // per subvolume
    std::vector<uint8_t> active;
    std::vector<BatchTile> tiles;       // current (active) tile list
    BatchSub* d_subs = nullptr;
    BatchTile* d_tiles = nullptr;
    int32_t* d_ntiles = nullptr;
    int32_t* d_counters = nullptr;      // one per step of a graph
    double* d_partial = nullptr;        // per tile
    int64_t max_tiles = 0;
    int32_t grid = 0, block = 256;
    cudaGraphExec_t graph = nullptr;
    int32_t graph_steps = 0;
    std::vector<int64_t> steps;         // per subvolume
    uint32_t seed_step = 0;             // steps taken since init (16-bit rounding seed)
};

static const uint32_t* seed_base(const LbmBatch* b) { return reinterpret_cast<const uint32_t*>(b->d_counters + 4096); }

namespace {
using namespace lbmk;

template <int STORE, bool FORCE, bool CHECK>
__global__ void __launch_bounds__(256, STORE == LBM_STORE_F64 ? 1 : 4) batch_step_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                                                         const BatchSub* __restrict__ subs,
                                                         const BatchTile* __restrict__ tiles,
                                                         const int32_t* __restrict__ n_tiles, int32_t* counter,
                                                         const typename Codec<STORE>::T* __restrict__ fin,
                                                         typename Codec<STORE>::T* __restrict__ fout,
                                                         const int32_t* __restrict__ map,
                                                         const uint32_t* __restrict__ coord,
                                                         const uint32_t* __restrict__ seed_base,
                                                         double* __restrict__ partial) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    __shared__ int s_tile;
    __shared__ double s_red[32];
    const int nt = *n_tiles;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
        __syncthreads();
        const int t = s_tile;
        __syncthreads();
        if (t >= nt) return;
        const BatchTile tl = tiles[t];
        const BatchSub sd = subs[tl.sub];
        const int32_t* smap = map + sd.map_off;
        const typename Cd::T* sfin = sub_pop(fin, sd.node_begin);
        typename Cd::T* sfout = sub_pop(fout, sd.node_begin);
        const uint32_t* scoord = coord + sd.node_begin;
        // 16-bit codecs: all faces periodic, so the reference density is 0; the
        // rounding bits are those of a single lattice at the same step (step
        // index = the launch group's first step, set before the group, + k)
        const uint32_t seed = *seed_base + C.seed;
        double acc = 0.0;
        for (int n = tl.begin + threadIdx.x; n < tl.end; n += blockDim.x) {
            const uint32_t pc = __ldg(scoord + n);
            const int i = lbm_pi(pc), j = lbm_pj(pc), k = lbm_pk(pc);
            R F[19];
            gather_node<STORE>(F, sfin, smap, n, sd.nx, sd.ny, sd.nz, i, j, k);
            R r = F[0];
#pragma unroll
            for (int s = 1; s < 19; ++s) r = r + F[s];
            const R rho = Cd::DEV ? (R)1 + r : r;
            R vx = vsum<0>(F) / rho, vy = vsum<1>(F) / rho, vz = vsum<2>(F) / rho;
            if constexpr (FORCE) {
                vx = vx + C.fhalf[0] / rho;
                vy = vy + C.fhalf[1] / rho;
                vz = vz + C.fhalf[2] / rho;
            }
            if constexpr (CHECK) acc += (double)vx;
            collide_sp<R, FORCE, Cd::DEV>(F, r, vx, vy, vz, C);
            store_node<STORE>(F, sfout, n, (R)0, seed);
        }
        if constexpr (CHECK) {
            for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
            if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double s = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += s_red[w];
                partial[t] = s;
            }
            __syncthreads();
        }
    }
}

// rho and v of one subvolume's nodes from its current populations (the
// macroscopic step of the next update, without collision or store).
template <int STORE, bool FORCE>
__global__ void batch_macros_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C, BatchSub sd,
                                    const typename Codec<STORE>::T* __restrict__ fin, const int32_t* __restrict__ map,
                                    const uint32_t* __restrict__ coord, float* __restrict__ out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= sd.n_fluid) return;
    const uint32_t pc = __ldg(coord + sd.node_begin + a);
    R F[19];
    gather_node<STORE>(F, sub_pop(fin, sd.node_begin), map + sd.map_off, a, sd.nx, sd.ny, sd.nz, lbm_pi(pc), lbm_pj(pc),
                       lbm_pk(pc));
    R r = F[0];
#pragma unroll
    for (int s = 1; s < 19; ++s) r = r + F[s];
    const R rho = Cd::DEV ? (R)1 + r : r;
    R vx = vsum<0>(F) / rho, vy = vsum<1>(F) / rho, vz = vsum<2>(F) / rho;
    if constexpr (FORCE) {
        vx = vx + C.fhalf[0] / rho;
        vy = vy + C.fhalf[1] / rho;
        vz = vz + C.fhalf[2] / rho;
    }
    out[4 * a] = (float)rho;
    out[4 * a + 1] = (float)vx;
    out[4 * a + 2] = (float)vy;
    out[4 * a + 3] = (float)vz;
}

template <int STORE, bool FORCE>
__global__ void batch_init_kernel(const __grid_constant__ SpConsts<typename Codec<STORE>::R> C,
                                  typename Codec<STORE>::T* __restrict__ fout, const BatchSub* __restrict__ subs,
                                  int n_sub) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    if (blockIdx.y >= (unsigned)n_sub) return;
    const BatchSub sd = subs[blockIdx.y];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= sd.n_fluid) return;
    R F[19];
    if constexpr (Cd::DEV) lbm_feq_dev_all<R>((R)0, (R)0, (R)0, (R)0, F);
    else lbm_feq_all<R>((R)1, (R)0, (R)0, (R)0, F);
    const R r = Cd::DEV ? (R)0 : (R)1;
    collide_sp<R, FORCE, Cd::DEV>(F, r, (R)0, (R)0, (R)0, C);
    store_node<STORE>(F, sub_pop(fout, sd.node_begin), n, (R)0, ~0u);   // as the single-lattice init
}

int batch_err(LbmBatch* b, int code, const std::string& m) { return lbm_set_err(&b->h, code, m); }

template <int STORE>
int launch_one(LbmBatch* b, int k, bool check, cudaStream_t s) {
    using Cd = Codec<STORE>;
    using T = typename Cd::T;
    using R = typename Cd::R;
    LbmHandle* h = &b->h;
    SpConsts<R> C = sp_make_consts<R>(h);
    C.seed = (uint32_t)k;   // step within the launch group; the group's first step is read on the device
    const int cur = k & 1;
    const T* fin = (const T*)h->d_f[cur];
    T* fout = (T*)h->d_f[cur ^ 1];
    int32_t* ctr = b->d_counters + k;
    auto args = [&](auto kern) {
        kern<<<b->grid, b->block, 0, s>>>(C, b->d_subs, b->d_tiles, b->d_ntiles, ctr, fin, fout, h->d_map, h->d_coord,
                                          seed_base(b), b->d_partial);
    };
    if (h->force) {
        if (check) args(batch_step_kernel<STORE, true, true>);
        else args(batch_step_kernel<STORE, true, false>);
    } else {
        if (check) args(batch_step_kernel<STORE, false, true>);
        else args(batch_step_kernel<STORE, false, false>);
    }
    return lbm_cuda_check(h, cudaGetLastError(), "batch_step_kernel launch");
}

int launch_dispatch(LbmBatch* b, int k, bool check, cudaStream_t s) {
    switch (b->h.p.storage) {
    case LBM_STORE_F32: return launch_one<LBM_STORE_F32>(b, k, check, s);
    case LBM_STORE_F16_DEV: return launch_one<LBM_STORE_F16_DEV>(b, k, check, s);
    case LBM_STORE_BF16_DEV: return launch_one<LBM_STORE_BF16_DEV>(b, k, check, s);
    case LBM_STORE_F32_DEV: return launch_one<LBM_STORE_F32_DEV>(b, k, check, s);
    case LBM_STORE_F64: return launch_one<LBM_STORE_F64>(b, k, check, s);
    }
    return batch_err(b, LBM_EINVAL, "unknown storage");
}

template <int STORE>
int occupancy(LbmBatch* b, int* per_sm) {
    // the CHECK variant has the same resource use; ask the runtime for the unforced and forced kernels
    const void* k = b->h.force ? (const void*)batch_step_kernel<STORE, true, false>
                               : (const void*)batch_step_kernel<STORE, false, false>;
    return lbm_cuda_check(&b->h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, b->block, 0), "occupancy");
}

int occ_dispatch(LbmBatch* b, int* per_sm) {
    switch (b->h.p.storage) {
    case LBM_STORE_F32: return occupancy<LBM_STORE_F32>(b, per_sm);
    case LBM_STORE_F16_DEV: return occupancy<LBM_STORE_F16_DEV>(b, per_sm);
    case LBM_STORE_BF16_DEV: return occupancy<LBM_STORE_BF16_DEV>(b, per_sm);
    case LBM_STORE_F32_DEV: return occupancy<LBM_STORE_F32_DEV>(b, per_sm);
    case LBM_STORE_F64: return occupancy<LBM_STORE_F64>(b, per_sm);
    }
    return batch_err(b, LBM_EINVAL, "unknown storage");
}

template <int STORE>
int init_t(LbmBatch* b) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    LbmHandle* h = &b->h;
    const SpConsts<R> C = sp_make_consts<R>(h);
    int maxn = 1;
    for (auto& s : b->subs) maxn = std::max(maxn, s.n_fluid);
    dim3 grid((maxn + 255) / 256, (unsigned)b->subs.size());
    auto k = h->force ? batch_init_kernel<STORE, true> : batch_init_kernel<STORE, false>;
    k<<<grid, 256, 0, h->stream>>>(C, (typename Cd::T*)h->d_f[0], b->d_subs, (int)b->subs.size());
    return lbm_cuda_check(h, cudaGetLastError(), "batch_init_kernel launch");
}

template <int STORE>
int macros_t(LbmBatch* b, int q, float* d_out) {
    using Cd = Codec<STORE>;
    using R = typename Cd::R;
    LbmHandle* h = &b->h;
    const SpConsts<R> C = sp_make_consts<R>(h);
    const BatchSub sd = b->subs[q];
    const int grid = (sd.n_fluid + 255) / 256;
    auto k = h->force ? batch_macros_kernel<STORE, true> : batch_macros_kernel<STORE, false>;
    if (grid > 0)
        k<<<grid, 256, 0, h->stream>>>(C, sd, (const typename Cd::T*)h->d_f[0], h->d_map, h->d_coord, d_out);
    return lbm_cuda_check(h, cudaGetLastError(), "batch_macros_kernel launch");
}

int rebuild_tiles(LbmBatch* b) {
    b->tiles.clear();
    for (size_t q = 0; q < b->subs.size(); ++q) {
        if (!b->active[q]) continue;
        const BatchSub& s = b->subs[q];
        const int len = std::max(32, b->tile_len[q]);
        for (int a = 0; a < s.n_fluid; a += len)
            b->tiles.push_back({(int32_t)q, a, std::min(s.n_fluid, a + len), 0});
    }
    LbmHandle* h = &b->h;
    if ((int64_t)b->tiles.size() > b->max_tiles) return batch_err(b, LBM_EINVAL, "tile list exceeds its allocation");
    const int32_t nt = (int32_t)b->tiles.size();
    int rc = 0;
    if (nt) rc = lbm_cuda_check(h, cudaMemcpyAsync(b->d_tiles, b->tiles.data(), sizeof(BatchTile) * nt, cudaMemcpyHostToDevice, h->stream), "copy tiles");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpyAsync(b->d_ntiles, &nt, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream), "copy ntiles");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "rebuild tiles");
    return rc;
}

void destroy_graph(LbmBatch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_steps = 0;
}

// Capture `nsteps` steps (the last one writes the per-tile partials) into a graph.
int capture(LbmBatch* b, int32_t nsteps) {
    LbmHandle* h = &b->h;
    destroy_graph(b);
    cudaGraph_t g;
    int rc = lbm_cuda_check(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (rc) return rc;
    cudaMemsetAsync(b->d_counters, 0, sizeof(int32_t) * nsteps, h->stream);
    for (int k = 0; k < nsteps && !rc; ++k) rc = launch_dispatch(b, k, k == nsteps - 1, h->stream);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) return rc;
    rc = lbm_cuda_check(h, e, "end capture");
    if (rc) return rc;
    rc = lbm_cuda_check(h, cudaGraphInstantiate(&b->graph, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    if (!rc) b->graph_steps = nsteps;
    return rc;
}

}  // namespace

extern "C" {

int lbm_batch_destroy(LbmBatch* b);

int lbm_batch_create(const LbmParams* params, int32_t n_sub, const int32_t* dims, const int8_t* solids,
                     LbmBatch** out) {
    if (!params || !dims || !solids || !out || n_sub < 1) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: bad argument");
    *out = nullptr;
    for (int f = 0; f < 6; ++f)
        if (params->bc[f] != 0) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: batched subvolumes are periodic on all faces");
    if (params->two_phase) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: single phase only");
    LbmParams p = *params;
    p.nx = p.ny = p.nz = 1;
    LbmHandle* tmp = nullptr;
    int rc = lbm_create(&p, &tmp);   // device checks, stream
    if (rc) return rc;
    LbmBatch* b = new LbmBatch();
    b->h = std::move(*tmp);
    tmp->stream = nullptr;
    lbm_destroy(tmp);
    LbmHandle* h = &b->h;
    // concatenate the subvolumes
    int64_t cells = 0, nodes = 0;
    std::vector<int32_t> map;
    std::vector<uint32_t> coord;
    for (int q = 0; q < n_sub; ++q) {
        const int nx = dims[3 * q], ny = dims[3 * q + 1], nz = dims[3 * q + 2];
        if (nx < 1 || ny < 1 || nz < 1 || nx > 2047 || ny > 2047 || nz > 1023) {
            lbm_batch_destroy(b);
            return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: bad subvolume size");
        }
        const int64_t nc = (int64_t)nx * ny * nz;
        BatchSub s{nx, ny, nz, 0, (int64_t)map.size(), nodes};
        const int8_t* sol = solids + cells;
        int64_t nf = 0;
        map.resize(map.size() + nc);
        for (int64_t c = 0; c < nc; ++c) {
            if (sol[c] > 0) { map[s.map_off + c] = -1; continue; }
            map[s.map_off + c] = (int32_t)nf;   // checked against the local limit below
            const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((int64_t)nx * ny));
            coord.push_back(lbm_pack(i, j, k));
            ++nf;
        }
        if (nf >= ((int64_t)1 << 31) / 19) {
            lbm_batch_destroy(b);
            return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: subvolume has too many fluid nodes");
        }
        s.n_fluid = (int32_t)nf;
        const int64_t padded = (nf + 31) / 32 * 32;
        coord.resize(coord.size() + (padded - nf), 0);
        nodes += padded;
        cells += nc;
        b->subs.push_back(s);
    }
    if (nodes >= ((int64_t)1 << 31) - 64) { lbm_batch_destroy(b); return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_create: too many nodes"); }
    h->n_fluid = (int32_t)nodes;
    h->np = (nodes + 63) / 64 * 64;
    coord.resize(h->np, 0);
    h->ncell = cells;
    b->active.assign(n_sub, 1);
    b->tile_len.assign(n_sub, 1024);
    b->steps.assign(n_sub, 0);
    b->max_tiles = 0;
    for (auto& s : b->subs) b->max_tiles += (s.n_fluid + 31) / 32;   // tiles of >= 32 nodes
    auto alloc = [&](void** ptr, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(ptr, bytes ? bytes : 16) != cudaSuccess) rc = lbm_set_err(nullptr, LBM_ENOMEM, "lbm_batch_create: out of device memory");
        else h->device_bytes += (int64_t)bytes;
    };
    alloc((void**)&h->d_map, sizeof(int32_t) * map.size());
    alloc((void**)&h->d_coord, sizeof(uint32_t) * h->np);
    alloc(&h->d_f[0], h->elem * 19 * h->np);
    alloc(&h->d_f[1], h->elem * 19 * h->np);
    alloc((void**)&b->d_subs, sizeof(BatchSub) * n_sub);
    alloc((void**)&b->d_tiles, sizeof(BatchTile) * b->max_tiles);
    alloc((void**)&b->d_ntiles, sizeof(int32_t));
    alloc((void**)&b->d_partial, sizeof(double) * b->max_tiles);
    alloc((void**)&b->d_counters, sizeof(int32_t) * (4096 + 4));   // + the first step of the launch group
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpy(h->d_map, map.data(), sizeof(int32_t) * map.size(), cudaMemcpyHostToDevice), "copy map");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpy(h->d_coord, coord.data(), sizeof(uint32_t) * h->np, cudaMemcpyHostToDevice), "copy coord");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpy(b->d_subs, b->subs.data(), sizeof(BatchSub) * n_sub, cudaMemcpyHostToDevice), "copy subs");
    if (rc) { lbm_batch_destroy(b); return rc; }
    h->have_geometry = true;
    *out = b;
    return LBM_OK;
}

int lbm_batch_destroy(LbmBatch* b) {
    if (!b) return LBM_OK;
    LbmHandle* h = &b->h;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    destroy_graph(b);
    cudaFree(b->d_subs);
    cudaFree(b->d_tiles);
    cudaFree(b->d_ntiles);
    cudaFree(b->d_partial);
    cudaFree(b->d_counters);
    cudaFree(h->d_map);
    cudaFree(h->d_coord);
    cudaFree(h->d_f[0]);
    cudaFree(h->d_f[1]);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete b;
    return LBM_OK;
}

// Tile length (nodes) per subvolume and threads per CTA of the persistent kernel.
int lbm_batch_configure(LbmBatch* b, const int32_t* tile_len, int32_t block) {
    if (!b || !tile_len) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_configure: NULL argument");
    if (block < 64 || block > 256 || block % 32) return batch_err(b, LBM_EINVAL, "lbm_batch_configure: block must be 64..256, multiple of 32");
    for (size_t q = 0; q < b->subs.size(); ++q) {
        if (tile_len[q] < 32) return batch_err(b, LBM_EINVAL, "lbm_batch_configure: tile length < 32");
        b->tile_len[q] = tile_len[q];
    }
    b->block = block;
    destroy_graph(b);
    return LBM_OK;
}

int lbm_batch_init(LbmBatch* b) {
    if (!b) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_init: NULL");
    LbmHandle* h = &b->h;
    cudaSetDevice(h->device);
    int per_sm = 0;
    int rc = occ_dispatch(b, &per_sm);
    if (rc) return rc;
    b->grid = std::max(1, per_sm) * h->sm_count;
    std::fill(b->active.begin(), b->active.end(), (uint8_t)1);
    std::fill(b->steps.begin(), b->steps.end(), (int64_t)0);
    switch (h->p.storage) {
    case LBM_STORE_F32: rc = init_t<LBM_STORE_F32>(b); break;
    case LBM_STORE_F16_DEV: rc = init_t<LBM_STORE_F16_DEV>(b); break;
    case LBM_STORE_BF16_DEV: rc = init_t<LBM_STORE_BF16_DEV>(b); break;
    case LBM_STORE_F32_DEV: rc = init_t<LBM_STORE_F32_DEV>(b); break;
    case LBM_STORE_F64: rc = init_t<LBM_STORE_F64>(b); break;
    default: rc = batch_err(b, LBM_EINVAL, "unknown storage");
    }
    if (!rc) rc = rebuild_tiles(b);
    b->seed_step = 0;
    destroy_graph(b);
    return rc;
}

// Step index of the next launch group's first step (rounding seed), written to
// the device before the group; advanced by the group's steps.
static int set_seed_base(LbmBatch* b, int32_t chunk) {
    const uint32_t v = b->seed_step;
    b->seed_step += (uint32_t)chunk;
    return lbm_cuda_check(&b->h, cudaMemcpyAsync(b->d_counters + 4096, &v, sizeof(v), cudaMemcpyHostToDevice, b->h.stream),
                          "seed base");
}

// Run `nsteps` (even) steps of all active subvolumes: graph launches of
// `chunk` steps when use_graph, else plain launches.  Leaves per-tile partials
// of the last step in device memory.
static int batch_run(LbmBatch* b, int32_t nsteps, int32_t chunk, int32_t use_graph) {
    LbmHandle* h = &b->h;
    if (use_graph) {
        if (b->graph_steps != chunk) {
            int rc = capture(b, chunk);
            if (rc) return rc;
        }
        for (int32_t done = 0; done < nsteps; done += chunk) {
            int rc = set_seed_base(b, chunk);
            if (!rc) rc = lbm_cuda_check(h, cudaGraphLaunch(b->graph, h->stream), "graph launch");
            if (rc) return rc;
        }
        return LBM_OK;
    }
    for (int32_t done = 0; done < nsteps; done += chunk) {
        int rc = set_seed_base(b, chunk);
        if (!rc) rc = lbm_cuda_check(h, cudaMemsetAsync(b->d_counters, 0, sizeof(int32_t) * chunk, h->stream), "counters");
        for (int k = 0; k < chunk && !rc; ++k) rc = launch_dispatch(b, k, k == chunk - 1, h->stream);
        if (rc) return rc;
    }
    return LBM_OK;
}

int lbm_batch_step(LbmBatch* b, int32_t nsteps, int32_t chunk, int32_t use_graph) {
    if (!b) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_step: NULL");
    if (chunk < 2 || chunk > 4096 || chunk % 2 || nsteps % chunk)
        return batch_err(b, LBM_EINVAL, "lbm_batch_step: chunk must be even, <= 4096, and divide nsteps");
    cudaSetDevice(b->h.device);
    int rc = batch_run(b, nsteps, chunk, use_graph);
    if (!rc) rc = lbm_cuda_check(&b->h, cudaStreamSynchronize(b->h.stream), "batch step");
    if (!rc)
        for (size_t q = 0; q < b->subs.size(); ++q)
            if (b->active[q]) b->steps[q] += nsteps;
    return rc;
}

// Darcy velocity along x of every active subvolume after the last step (the
// sum of v_x over its fluid nodes / its cells); inactive ones keep their value.
static int batch_darcy(LbmBatch* b, double* darcy) {
    LbmHandle* h = &b->h;
    std::vector<double> part(b->tiles.size());
    int rc = 0;
    if (!part.empty())
        rc = lbm_cuda_check(h, cudaMemcpy(part.data(), b->d_partial, sizeof(double) * part.size(), cudaMemcpyDeviceToHost), "copy partials");
    if (rc) return rc;
    std::vector<double> sum(b->subs.size(), 0.0);
    for (size_t t = 0; t < b->tiles.size(); ++t) sum[b->tiles[t].sub] += part[t];
    for (size_t q = 0; q < b->subs.size(); ++q)
        if (b->active[q]) {
            const BatchSub& s = b->subs[q];
            darcy[q] = sum[q] / ((double)s.nx * s.ny * s.nz);
        }
    return LBM_OK;
}

int lbm_batch_run_to_convergence(LbmBatch* b, double tol, int32_t check_every, int64_t max_steps, int32_t use_graph,
                                 double* darcy, int64_t* steps, int32_t* converged) {
    if (!b || !darcy || !steps || !converged) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_run_to_convergence: NULL");
    if (check_every < 2 || check_every > 4096 || check_every % 2)
        return batch_err(b, LBM_EINVAL, "lbm_batch_run_to_convergence: check_every must be even and <= 4096");
    LbmHandle* h = &b->h;
    cudaSetDevice(h->device);
    const size_t ns = b->subs.size();
    std::vector<double> prev(ns, 0.0), cur(ns, 0.0);
    std::vector<uint8_t> have(ns, 0);
    for (size_t q = 0; q < ns; ++q) converged[q] = 0;
    int64_t done = 0;
    while (done < max_steps) {
        bool any = false;
        for (size_t q = 0; q < ns; ++q) any |= b->active[q] != 0;
        if (!any) break;
        int rc = batch_run(b, check_every, check_every, use_graph);
        if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "batch run");
        if (rc) return rc;
        done += check_every;
        for (size_t q = 0; q < ns; ++q)
            if (b->active[q]) b->steps[q] += check_every;
        rc = batch_darcy(b, cur.data());
        if (rc) return rc;
        bool changed = false;
        for (size_t q = 0; q < ns; ++q) {
            if (!b->active[q]) continue;
            if (!std::isfinite(cur[q])) return batch_err(b, LBM_EDIVERGED, "subvolume diverged");
            if (have[q] && std::fabs(cur[q] - prev[q]) <= tol * std::fabs(cur[q])) {
                b->active[q] = 0;
                converged[q] = 1;
                changed = true;
            }
            prev[q] = cur[q];
            have[q] = 1;
        }
        if (changed) {
            rc = rebuild_tiles(b);
            if (rc) return rc;
        }
    }
    for (size_t q = 0; q < ns; ++q) {
        darcy[q] = cur[q];
        steps[q] = b->steps[q];
    }
    return LBM_OK;
}

int lbm_batch_get_macros(LbmBatch* b, int32_t sub, float* rho, float* v) {
    if (!b || !rho || !v) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_get_macros: NULL");
    if (sub < 0 || sub >= (int32_t)b->subs.size()) return batch_err(b, LBM_EINVAL, "lbm_batch_get_macros: bad subvolume");
    LbmHandle* h = &b->h;
    cudaSetDevice(h->device);
    const BatchSub sd = b->subs[sub];
    float* d_out = nullptr;
    if (cudaMalloc((void**)&d_out, sizeof(float) * 4 * std::max(1, sd.n_fluid)) != cudaSuccess)
        return batch_err(b, LBM_ENOMEM, "lbm_batch_get_macros: out of device memory");
    int rc = 0;
    switch (h->p.storage) {
    case LBM_STORE_F32: rc = macros_t<LBM_STORE_F32>(b, sub, d_out); break;
    case LBM_STORE_F16_DEV: rc = macros_t<LBM_STORE_F16_DEV>(b, sub, d_out); break;
    case LBM_STORE_BF16_DEV: rc = macros_t<LBM_STORE_BF16_DEV>(b, sub, d_out); break;
    case LBM_STORE_F32_DEV: rc = macros_t<LBM_STORE_F32_DEV>(b, sub, d_out); break;
    case LBM_STORE_F64: rc = macros_t<LBM_STORE_F64>(b, sub, d_out); break;
    }
    std::vector<float> tmp(4 * (size_t)sd.n_fluid);
    if (!rc && sd.n_fluid)
        rc = lbm_cuda_check(h, cudaMemcpyAsync(tmp.data(), d_out, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, h->stream), "copy macros");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "batch macros");
    cudaFree(d_out);
    if (rc) return rc;
    // scatter to the dense lattice (solid: rho = 1, v = 0) through the host copy of the map
    const int64_t nc = (int64_t)sd.nx * sd.ny * sd.nz;
    std::vector<int32_t> map(nc);
    rc = lbm_cuda_check(h, cudaMemcpy(map.data(), h->d_map + sd.map_off, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost), "copy map");
    if (rc) return rc;
    for (int64_t c = 0; c < nc; ++c) {
        const int32_t nd = map[c];
        if (nd < 0) {
            rho[c] = 1.0f;
            v[3 * c] = v[3 * c + 1] = v[3 * c + 2] = 0.0f;
        } else {
            const int64_t a = nd;
            rho[c] = tmp[4 * a];
            for (int d = 0; d < 3; ++d) v[3 * c + d] = tmp[4 * a + 1 + d];
        }
    }
    return LBM_OK;
}

int lbm_batch_get_stream(LbmBatch* b, void** stream) {
    if (!b || !stream) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_get_stream: NULL");
    *stream = (void*)b->h.stream;
    return LBM_OK;
}

int lbm_batch_info(LbmBatch* b, int64_t* n_nodes, int64_t* n_fluid, int32_t* grid, int32_t* n_tiles) {
    if (!b) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_batch_info: NULL");
    int64_t nf = 0;
    for (auto& s : b->subs) nf += s.n_fluid;
    if (n_nodes) *n_nodes = b->h.n_fluid;
    if (n_fluid) *n_fluid = nf;
    if (grid) *grid = b->grid;
    if (n_tiles) *n_tiles = (int32_t)b->tiles.size();
    return LBM_OK;
}

}  // extern "C"
