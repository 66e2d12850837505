// K3: FP64 reductions over the fluid nodes of the last step: mass (sum rho),
// momentum sums (sum v), max |v| (get_max_v / cal_max_v, SP:394-402, where the
// norm is the FP32 sqrt of the FP32 dot product) and a count of non-finite
// values.  Two passes (per-block partials, then one block), fixed summation
// order: results are identical run to run.
#include <cuda_runtime.h>

#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace {

constexpr int RED_THREADS = 256;
constexpr int RED_FIELDS = 6;  // mass, mx, my, mz, max|v|, nonfinite

template <typename R>
__device__ __forceinline__ void red_node(const R* __restrict__ rho, const R* __restrict__ v, int64_t np, int n,
                                         double acc[RED_FIELDS]) {
    const R r = rho[n], vx = v[n], vy = v[np + n], vz = v[2 * np + n];
    const R nrm = sqrt(lbm_usq(vx, vy, vz));
    const bool fin = isfinite(r) && isfinite(vx) && isfinite(vy) && isfinite(vz);
    acc[0] += (double)r;
    acc[1] += (double)vx;
    acc[2] += (double)vy;
    acc[3] += (double)vz;
    acc[4] = fmax(acc[4], (double)nrm);
    acc[5] += fin ? 0.0 : 1.0;
}

__device__ __forceinline__ void red_combine(double a[RED_FIELDS], const double b[RED_FIELDS]) {
    for (int q = 0; q < 4; ++q) a[q] += b[q];
    a[4] = fmax(a[4], b[4]);
    a[5] += b[5];
}

// Block-wide reduction of RED_FIELDS doubles; result valid in thread 0.
__device__ void block_reduce(double acc[RED_FIELDS]) {
    __shared__ double sh[RED_THREADS / 32][RED_FIELDS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        double o[RED_FIELDS];
        for (int q = 0; q < RED_FIELDS; ++q) o[q] = __shfl_down_sync(0xffffffffu, acc[q], off);
        red_combine(acc, o);
    }
    if (lane == 0)
        for (int q = 0; q < RED_FIELDS; ++q) sh[wid][q] = acc[q];
    __syncthreads();
    if (wid == 0) {
        for (int q = 0; q < RED_FIELDS; ++q) acc[q] = lane < RED_THREADS / 32 ? sh[lane][q] : (q == 4 ? 0.0 : 0.0);
        for (int off = 16; off > 0; off >>= 1) {
            double o[RED_FIELDS];
            for (int q = 0; q < RED_FIELDS; ++q) o[q] = __shfl_down_sync(0xffffffffu, acc[q], off);
            red_combine(acc, o);
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) red_partial_kernel(const R* __restrict__ rho, const R* __restrict__ v,
                                                                  int64_t np, int n_fluid, double* __restrict__ part) {
    double acc[RED_FIELDS] = {0, 0, 0, 0, 0, 0};
    for (int n = blockIdx.x * RED_THREADS + threadIdx.x; n < n_fluid; n += gridDim.x * RED_THREADS)
        red_node<R>(rho, v, np, n, acc);
    block_reduce(acc);
    if (threadIdx.x == 0)
        for (int q = 0; q < RED_FIELDS; ++q) part[blockIdx.x * RED_FIELDS + q] = acc[q];
}

__global__ void __launch_bounds__(RED_THREADS) red_final_kernel(const double* __restrict__ part, int nb,
                                                                double* __restrict__ out) {
    double acc[RED_FIELDS] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += RED_THREADS) red_combine(acc, part + b * RED_FIELDS);
    block_reduce(acc);
    if (threadIdx.x == 0)
        for (int q = 0; q < RED_FIELDS; ++q) out[q] = acc[q];
}

}  // namespace

int red_launch(LbmHandle* h, LbmStats* out, float* max_v_f32) {
    const int nb = h->red_blocks;
    if (h->f64)
        red_partial_kernel<double><<<nb, RED_THREADS, 0, h->stream>>>((const double*)h->d_rho, (const double*)h->d_v,
                                                                       h->np, h->n_fluid, h->d_red);
    else
        red_partial_kernel<float><<<nb, RED_THREADS, 0, h->stream>>>((const float*)h->d_rho, (const float*)h->d_v,
                                                                      h->np, h->n_fluid, h->d_red);
    int rc = lbm_cuda_check(h, cudaGetLastError(), "red_partial_kernel launch");
    if (rc) return rc;
    red_final_kernel<<<1, RED_THREADS, 0, h->stream>>>(h->d_red, nb, h->d_red_out);
    rc = lbm_cuda_check(h, cudaGetLastError(), "red_final_kernel launch");
    if (rc) return rc;
    double res[RED_FIELDS];
    rc = lbm_cuda_check(h, cudaMemcpyAsync(res, h->d_red_out, sizeof(res), cudaMemcpyDeviceToHost, h->stream), "copy reduction");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "reduction");
    if (rc) return rc;
    out->mass = res[0];
    out->mom[0] = res[1];
    out->mom[1] = res[2];
    out->mom[2] = res[3];
    out->max_v = res[4];
    out->n_nonfinite = (int64_t)res[5];
    out->n_fluid = h->n_fluid;
    if (max_v_f32) *max_v_f32 = (float)res[4];
    return LBM_OK;
}
