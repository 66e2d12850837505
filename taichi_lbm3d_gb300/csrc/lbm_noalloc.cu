// lbm_reduce_macros_noalloc: the FP64 macro reduction for callers that cannot
// allocate device memory.
//
// Who needs it: code that embeds this library inside a host framework whose
// own pool allocator already owns the device memory (so a cudaMalloc here
// would fail or fight that pool), and code driving time-critical work on other
// streams that cannot afford the device-wide synchronisation that cudaMalloc /
// cudaFree can trigger.  Such a caller passes its own device arrays of rho and v
// (node order, FP32) and receives the sums on the host; nothing is allocated.
//
// How: the per-block partial sums live in g_noalloc_scratch, a file-scope
// static __device__ array.  Every GPU that loads this library holds it
// (LBM_NOALLOC_SCRATCH_BYTES) until the process exits.  In host code the
// symbol is only a host-side stand-in, never a device address, so the device
// address is fetched with cudaGetSymbolAddress, with the device current, on the
// first call made on that device (make that first call before any stream
// capture begins) and cached together with the unique ID of the CUDA context it
// belongs to.  A later call that finds another context current on the device
// (the caller ran cudaDeviceReset, or the primary context was released and
// created again, which reloads this module and can move the array) looks the
// address up again instead of using the stale one.  The call is synchronous:
// it waits for its stream and returns the sums in host memory.
//
// Every call shares the one array and leaves its partials in it.  Each call
// writes every slot it later reads (one per block, then the result slots), so
// nothing has to be cleared between calls; calls that overlap on the GPU (two
// streams, two host threads) race on the array and must be serialised by the
// caller.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace {
constexpr int NA_THREADS = 256;
constexpr int NA_FIELDS = 6;                          // mass, mx, my, mz, max|v|, non-finite
constexpr int64_t NA_CHUNK = 256 * 64;                // nodes per block
constexpr int NA_MAX_BLOCKS = LBM_NOALLOC_MAX_NODES / NA_CHUNK;
static_assert((int64_t)NA_MAX_BLOCKS * NA_CHUNK == LBM_NOALLOC_MAX_NODES, "limit must be whole blocks");
constexpr int NA_RESULT = NA_MAX_BLOCKS * NA_FIELDS;  // offset of the final result
}  // namespace

// Partials of up to NA_MAX_BLOCKS blocks plus the result: 196,656 bytes.
static __device__ __align__(256) double g_noalloc_scratch[(NA_MAX_BLOCKS + 1) * NA_FIELDS];
static_assert(sizeof(g_noalloc_scratch) == LBM_NOALLOC_SCRATCH_BYTES, "header states the scratch size");

namespace {

__device__ __forceinline__ void na_combine(double a[NA_FIELDS], const double b[NA_FIELDS]) {
    for (int q = 0; q < 4; ++q) a[q] += b[q];
    a[4] = fmax(a[4], b[4]);
    a[5] += b[5];
}

__device__ void na_block_reduce(double acc[NA_FIELDS]) {
    __shared__ double sh[NA_THREADS / 32][NA_FIELDS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        double o[NA_FIELDS];
        for (int q = 0; q < NA_FIELDS; ++q) o[q] = __shfl_down_sync(0xffffffffu, acc[q], off);
        na_combine(acc, o);
    }
    if (lane == 0)
        for (int q = 0; q < NA_FIELDS; ++q) sh[wid][q] = acc[q];
    __syncthreads();
    if (wid == 0) {
        for (int q = 0; q < NA_FIELDS; ++q) acc[q] = lane < NA_THREADS / 32 ? sh[lane][q] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            double o[NA_FIELDS];
            for (int q = 0; q < NA_FIELDS; ++q) o[q] = __shfl_down_sync(0xffffffffu, acc[q], off);
            na_combine(acc, o);
        }
    }
}

// Block b reduces nodes [b*NA_CHUNK, min(n, (b+1)*NA_CHUNK)) into scratch[b].
__global__ void __launch_bounds__(NA_THREADS) na_partial_kernel(const float* __restrict__ rho,
                                                                const float* __restrict__ v, int64_t n,
                                                                int64_t stride, double* __restrict__ scratch) {
    double acc[NA_FIELDS] = {0, 0, 0, 0, 0, 0};
    const int64_t lo = (int64_t)blockIdx.x * NA_CHUNK;
    const int64_t hi = lo + NA_CHUNK < n ? lo + NA_CHUNK : n;
    for (int64_t i = lo + threadIdx.x; i < hi; i += NA_THREADS) {
        const float r = rho[i], vx = v[i], vy = v[stride + i], vz = v[2 * stride + i];
        const float nrm = sqrtf(lbm_usq(vx, vy, vz));
        acc[0] += (double)r;
        acc[1] += (double)vx;
        acc[2] += (double)vy;
        acc[3] += (double)vz;
        acc[4] = fmax(acc[4], (double)nrm);
        acc[5] += (isfinite(r) && isfinite(vx) && isfinite(vy) && isfinite(vz)) ? 0.0 : 1.0;
    }
    na_block_reduce(acc);
    if (threadIdx.x == 0)
        for (int q = 0; q < NA_FIELDS; ++q) scratch[(int64_t)blockIdx.x * NA_FIELDS + q] = acc[q];
}

__global__ void __launch_bounds__(NA_THREADS) na_final_kernel(double* __restrict__ scratch, int nb) {
    double acc[NA_FIELDS] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += NA_THREADS) na_combine(acc, scratch + (int64_t)b * NA_FIELDS);
    na_block_reduce(acc);
    if (threadIdx.x == 0)
        for (int q = 0; q < NA_FIELDS; ++q) scratch[NA_RESULT + q] = acc[q];
}

std::mutex g_na_mu;
struct NaScratch {
    double* ptr = nullptr;
    unsigned long long ctx_id = 0;   // context the address belongs to
    bool valid = false;
};
NaScratch g_na_dev[64];

// Driver entry points, resolved through the runtime (no link against libcuda).
typedef CUresult(CUDAAPI* NaCtxGetCurrent)(CUcontext*);
typedef CUresult(CUDAAPI* NaCtxGetId)(CUcontext, unsigned long long*);
NaCtxGetCurrent g_na_get_current = nullptr;
NaCtxGetId g_na_get_id = nullptr;
std::once_flag g_na_once;

// Unique ID of the context current on this thread; false when it cannot be
// known (no context yet, or the driver entry points are unavailable).
bool na_context_id(unsigned long long* id) {
    std::call_once(g_na_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_na_get_current = (NaCtxGetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_na_get_id = (NaCtxGetId)f;
    });
    if (!g_na_get_current || !g_na_get_id) return false;
    CUcontext ctx = nullptr;
    if (g_na_get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return g_na_get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of g_noalloc_scratch on the current device: looked up on the
// first call on a device and again whenever the current context differs from
// the one the cached address was taken in (every call, if the context ID
// cannot be read).
int na_scratch(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("lbm_reduce_macros_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_reduce_macros_noalloc: device ordinal >= 64");
    std::lock_guard<std::mutex> lk(g_na_mu);
    unsigned long long id = 0;
    NaScratch& c = g_na_dev[dev];
    if (c.valid && na_context_id(&id) && id == c.ctx_id) {
        *out = c.ptr;
        return LBM_OK;
    }
    c.valid = false;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);     // makes the device's primary context current if none is
    if (e != cudaSuccess || p == nullptr)
        return lbm_set_err(nullptr, LBM_ECUDA, std::string("lbm_reduce_macros_noalloc: cudaGetSymbolAddress: ") +
                                                   cudaGetErrorString(e));
    c.ptr = (double*)p;
    c.valid = na_context_id(&c.ctx_id);
    *out = c.ptr;
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_reduce_macros_noalloc(const float* rho, const float* v, int64_t n, int64_t v_stride, void* stream,
                                         LbmStats* out) {
    if (!out) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_reduce_macros_noalloc: out is NULL");
    if (n < 0) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_reduce_macros_noalloc: negative node count");
    if (n > LBM_NOALLOC_MAX_NODES) {
        char b[200];
        std::snprintf(b, sizeof b,
                      "lbm_reduce_macros_noalloc: n = %lld nodes exceeds the static scratch limit of %d nodes "
                      "(LBM_NOALLOC_MAX_NODES); use lbm_reductions on a handle instead",
                      (long long)n, (int)LBM_NOALLOC_MAX_NODES);
        return lbm_set_err(nullptr, LBM_EINVAL, b);
    }
    out->mass = 0;
    out->mom[0] = out->mom[1] = out->mom[2] = 0;
    out->max_v = 0;
    out->n_nonfinite = 0;
    out->n_fluid = n;
    if (n == 0) return LBM_OK;
    if (!rho || !v) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_reduce_macros_noalloc: rho or v is NULL");
    if (v_stride < n) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_reduce_macros_noalloc: v_stride < n");
    double* scratch = nullptr;
    int rc = na_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (int)((n + NA_CHUNK - 1) / NA_CHUNK);
    na_partial_kernel<<<nb, NA_THREADS, 0, s>>>(rho, v, n, v_stride, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        na_final_kernel<<<1, NA_THREADS, 0, s>>>(scratch, nb);
        e = cudaGetLastError();
    }
    double res[NA_FIELDS];
    if (e == cudaSuccess) e = cudaMemcpyAsync(res, scratch + NA_RESULT, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, std::string("lbm_reduce_macros_noalloc: ") + cudaGetErrorString(e));
    out->mass = res[0];
    out->mom[0] = res[1];
    out->mom[1] = res[2];
    out->mom[2] = res[3];
    out->max_v = res[4];
    out->n_nonfinite = (int64_t)res[5];
    return LBM_OK;
}
