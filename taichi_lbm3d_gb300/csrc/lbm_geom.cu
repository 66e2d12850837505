// Lattice index construction and dense output on the GPU.
//
// The compacted index (fluid nodes in cell order, x fastest: the order in which
// the reference's block-sparse storage is activated by init, SP:160-170) is
// built from the solid mask in three launches: per-tile fluid counts (1024
// cells per tile), one exclusive scan over the tiles, and a write pass that
// ranks each fluid cell inside its tile and stores map[cell] (node or -1) and
// the packed coordinates of each node.  The mask is read through element
// strides, so a C-ordered (z fastest) numpy array needs no host-side
// transposition.  Host copies of the index (solid flags, cell of each node) are
// made only when a host-side caller needs them.
//
// Dense output: one pass over the cells writes node values (or the solid fill)
// into a stream-ordered device buffer that is then copied to the caller.
// SP = Single_phase/LBM_3D_SinglePhase_Solver.py (taichi_LBM3D tree).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace {
constexpr int GEO_THREADS = 256;
constexpr int GEO_PER_THREAD = 4;
constexpr int GEO_TILE = GEO_THREADS * GEO_PER_THREAD;

struct MaskView {
    const int8_t* p;
    int64_t si, sj, sk;
    int nx, ny;
    int32_t ncell;
};

__device__ __forceinline__ bool cell_fluid(const MaskView& m, int32_t c) {
    const int i = c % m.nx, j = (c / m.nx) % m.ny, k = c / (m.nx * m.ny);
    return m.p[i * m.si + j * m.sj + k * m.sk] <= 0;   // solid > 0 (init_geo, SP:173-177)
}

// Exclusive prefix of v over the block; returns the block total in *total.
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int s_warp[GEO_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < GEO_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < GEO_THREADS / 32) s_warp[lane] = w;   // inclusive warp totals
    }
    __syncthreads();
    const int before = warp ? s_warp[warp - 1] : 0;
    *total = s_warp[GEO_THREADS / 32 - 1];
    return before + x - v;
}

__global__ void __launch_bounds__(GEO_THREADS) geo_count_kernel(const MaskView m, int32_t* __restrict__ tile_count) {
    const int32_t base = blockIdx.x * GEO_TILE + threadIdx.x * GEO_PER_THREAD;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < GEO_PER_THREAD; ++q)
        if (base + q < m.ncell && cell_fluid(m, base + q)) ++cnt;
    int total;
    block_exclusive_scan(cnt, &total);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

// One block: exclusive scan of the tile counts in place; the grand total (64-bit) to *sum.
__global__ void __launch_bounds__(1024) geo_scan_kernel(int32_t* __restrict__ tiles, int32_t ntiles, int64_t* __restrict__ sum) {
    __shared__ int64_t s_part[1024];
    const int t = threadIdx.x;
    const int per = (ntiles + 1023) / 1024;
    const int a = t * per, b = min(ntiles, a + per);
    int64_t local = 0;
    for (int q = a; q < b; ++q) local += tiles[q];
    s_part[t] = local;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {   // inclusive Hillis-Steele scan of the chunk sums
        const int64_t y = t >= o ? s_part[t - o] : 0;
        __syncthreads();
        s_part[t] += y;
        __syncthreads();
    }
    int64_t run = s_part[t] - local;
    for (int q = a; q < b; ++q) {
        const int32_t c = tiles[q];
        tiles[q] = (int32_t)run;     // the caller rejects totals >= 2^31 before using the offsets
        run += c;
    }
    if (t == 1023) *sum = s_part[1023];
}

__global__ void __launch_bounds__(GEO_THREADS) geo_write_kernel(const MaskView m, const int32_t* __restrict__ tile_off,
                                                               int32_t* __restrict__ map, uint32_t* __restrict__ coord) {
    const int32_t base = blockIdx.x * GEO_TILE + threadIdx.x * GEO_PER_THREAD;
    bool fl[GEO_PER_THREAD];
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < GEO_PER_THREAD; ++q) {
        fl[q] = base + q < m.ncell && cell_fluid(m, base + q);
        cnt += fl[q];
    }
    int total;
    int node = tile_off[blockIdx.x] + block_exclusive_scan(cnt, &total);
#pragma unroll
    for (int q = 0; q < GEO_PER_THREAD; ++q) {
        const int32_t c = base + q;
        if (c >= m.ncell) break;
        if (fl[q]) {
            map[c] = node;
            coord[node] = lbm_pack(c % m.nx, (c / m.nx) % m.ny, c / (m.nx * m.ny));
            ++node;
        } else {
            map[c] = -1;
        }
    }
}

// out[c*comps + d] = node value d of cell c, or fill for solid cells.
template <typename S, typename O>
__global__ void dense_out_kernel(const int32_t* __restrict__ map, const S* __restrict__ src, int64_t np, int comps,
                                 int64_t ncell, O fill, O* __restrict__ out) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int32_t n = map[c];
    for (int d = 0; d < comps; ++d) out[c * comps + d] = n >= 0 ? (O)src[d * np + n] : fill;
}
}  // namespace

// Build map and coordinates on the device from a mask addressed as
// solid[i*si + j*sj + k*sk]; allocates d_map and d_coord and sets n_fluid, np.
int geom_build(LbmHandle* h, const int8_t* solid, int64_t si, int64_t sj, int64_t sk) {
    const int nx = h->p.nx, ny = h->p.ny, nz = h->p.nz;
    const int64_t ncell = h->ncell;
    const int64_t span = (int64_t)(nx - 1) * si + (int64_t)(ny - 1) * sj + (int64_t)(nz - 1) * sk + 1;
    const int32_t ntiles = (int32_t)((ncell + GEO_TILE - 1) / GEO_TILE);
    int8_t* d_mask = nullptr;
    int32_t* d_tiles = nullptr;
    int64_t* d_sum = nullptr;
    cudaStream_t st = h->stream;
    int rc = lbm_cuda_check(h, cudaMallocAsync((void**)&d_mask, (size_t)span, st), "geometry staging");
    if (!rc) rc = lbm_cuda_check(h, cudaMallocAsync((void**)&d_tiles, sizeof(int32_t) * ntiles, st), "geometry tiles");
    if (!rc) rc = lbm_cuda_check(h, cudaMallocAsync((void**)&d_sum, sizeof(int64_t), st), "geometry total");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpyAsync(d_mask, solid, (size_t)span, cudaMemcpyHostToDevice, st), "copy mask");
    const MaskView m{d_mask, si, sj, sk, nx, ny, (int32_t)ncell};
    int64_t total = 0;
    if (!rc) {
        geo_count_kernel<<<ntiles, GEO_THREADS, 0, st>>>(m, d_tiles);
        geo_scan_kernel<<<1, 1024, 0, st>>>(d_tiles, ntiles, d_sum);
        rc = lbm_cuda_check(h, cudaGetLastError(), "geometry scan launch");
    }
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpyAsync(&total, d_sum, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "copy total");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(st), "geometry count");
    // 32-bit population offsets: element (n, s) sits at about 19 n (lbm_eoff32)
    if (!rc && total >= ((int64_t)1 << 31) / 19 - 64)
        rc = lbm_set_err(h, LBM_EINVAL, "lbm_set_geometry: " + std::to_string(total) +
                                           " fluid nodes; one lattice holds fewer than 2^31/19 (split it into a batch)");
    if (!rc) {
        h->n_fluid = (int32_t)total;
        h->np = (std::max<int64_t>(total, 1) + 63) / 64 * 64;
        // LBM_MAP_PAD entries of -1 after the last cell: the step kernel stages map
        // rows with 16-byte bulk copies, which may round a row block up past its end
        rc = lbm_cuda_check(h, cudaMalloc((void**)&h->d_map, sizeof(int32_t) * (ncell + LBM_MAP_PAD)), "map");
        if (!rc) h->device_bytes += sizeof(int32_t) * (ncell + LBM_MAP_PAD);
        if (!rc)
            rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_map + ncell, 0xff, sizeof(int32_t) * LBM_MAP_PAD, st),
                                "map padding");
        if (!rc) rc = lbm_cuda_check(h, cudaMalloc((void**)&h->d_coord, sizeof(uint32_t) * h->np), "coord");
        if (!rc) h->device_bytes += sizeof(uint32_t) * h->np;
        if (!rc) rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_coord, 0, sizeof(uint32_t) * h->np, st), "clear coord");
    }
    if (!rc) {
        geo_write_kernel<<<ntiles, GEO_THREADS, 0, st>>>(m, d_tiles, h->d_map, h->d_coord);
        rc = lbm_cuda_check(h, cudaGetLastError(), "geometry write launch");
    }
    if (d_mask) cudaFreeAsync(d_mask, st);
    if (d_tiles) cudaFreeAsync(d_tiles, st);
    if (d_sum) cudaFreeAsync(d_sum, st);
    h->host_index_valid = false;
    return rc;
}

// Host copies of the index (solid flags per cell, cell of each node), made on demand.
int geom_host_index(LbmHandle* h) {
    if (h->host_index_valid) return LBM_OK;
    std::vector<int32_t> map(h->ncell);
    int rc = lbm_cuda_check(h, cudaMemcpyAsync(map.data(), h->d_map, sizeof(int32_t) * h->ncell, cudaMemcpyDeviceToHost, h->stream), "copy map");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "copy map");
    if (rc) return rc;
    h->solid.assign(h->ncell, 0);
    h->cell_of_node.assign(h->n_fluid, 0);
    for (int64_t c = 0; c < h->ncell; ++c) {
        const int32_t n = map[c];
        if (n < 0) h->solid[c] = 1;
        else h->cell_of_node[n] = (int32_t)c;
    }
    h->host_index_valid = true;
    return LBM_OK;
}

// Dense host array (comps interleaved per cell) from a node-ordered device
// array (comps components of stride np, the handle's compute type).
template <typename O>
int geom_dense_out(LbmHandle* h, const void* dsrc, int comps, O* out, O fill) {
    const int64_t n = h->ncell * comps;
    O* d_out = nullptr;
    int rc = lbm_cuda_check(h, cudaMallocAsync((void**)&d_out, sizeof(O) * n, h->stream), "output staging");
    if (rc) return rc;
    const int blocks = (int)((h->ncell + 255) / 256);
    if (h->f64)
        dense_out_kernel<double, O><<<blocks, 256, 0, h->stream>>>(h->d_map, (const double*)dsrc, h->np, comps, h->ncell, fill, d_out);
    else
        dense_out_kernel<float, O><<<blocks, 256, 0, h->stream>>>(h->d_map, (const float*)dsrc, h->np, comps, h->ncell, fill, d_out);
    rc = lbm_cuda_check(h, cudaGetLastError(), "dense_out_kernel launch");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpyAsync(out, d_out, sizeof(O) * n, cudaMemcpyDeviceToHost, h->stream), "copy out");
    cudaFreeAsync(d_out, h->stream);
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "copy out");
    return rc;
}
template int geom_dense_out<float>(LbmHandle*, const void*, int, float*, float);
template int geom_dense_out<double>(LbmHandle*, const void*, int, double*, double);
