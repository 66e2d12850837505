// Kernels of the warm-start network (a 3-level 3D U-Net, see unet.py):
// 3x3x3 convolutions, 2x max-pool, 2x nearest upsample, channel concat/split,
// 1x1 output head, masked MSE, Adam.  Activations are BF16, channels last
// (N, D, H, W, C); accumulation is FP32.
//
// The 3x3x3 convolution (forward, backward data) and its weight gradient run
// on the tcgen05 tensor cores (nn_tc.cu); the weight gradient leaves one FP32
// partial per (voxel chunk, tap), summed here in a fixed order.
#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/lbm_nn.h"
#include "lbm_internal.h"
#include "nn_act.cuh"

// tensor-core weight gradient (nn_tc.cu)
int nn_wgrad_tc_launch(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int w, int cin,
                       int cout, cudaStream_t s);
int64_t nn_wgrad_tc_chunks(int64_t nvox);

namespace {

typedef __nv_bfloat16 bf16;

struct Vox {
    int n, z, y, x;
};

__device__ __forceinline__ Vox decode(int64_t v, int D, int H, int W) {
    Vox o;
    o.x = (int)(v % W);
    int64_t t = v / W;
    o.y = (int)(t % H);
    t /= H;
    o.z = (int)(t % D);
    o.n = (int)(t / D);
    return o;
}

// dw[co][tap][ci] = sum over chunks (fixed order) of part[chunk][tap][co][ci].
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const float* __restrict__ part, float* __restrict__ dw,
                                                            int nchunk, int cin, int cout) {
    // 32 consecutive elements per CTA (one 128-byte row per chunk); warp w sums chunks w, w + 8, ...
    // in that order, then the 8 warp sums are added in warp order: a fixed order for any launch
    __shared__ float s_part[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t total = (int64_t)27 * cout * cin;
    const int64_t e = (int64_t)blockIdx.x * 32 + lane;
    float s = 0.f;
    if (e < total) {
#pragma unroll 8
        for (int c = warp; c < nchunk; c += 8) s += part[(int64_t)c * total + e];
    }
    s_part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && e < total) {
        float t = 0.f;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += s_part[w][lane];
        const int tap = (int)(e / ((int64_t)cout * cin));
        const int co = (int)((e / cin) % cout), ci = (int)(e % cin);
        dw[((int64_t)co * 27 + tap) * cin + ci] = t;
    }
}

// db[co] = sum over chunks of dbpart[chunk][co], in the same fixed warp-split order.
__global__ void __launch_bounds__(256) bias_reduce_kernel(const float* __restrict__ dbpart, float* __restrict__ db,
                                                           int nchunk, int cout) {
    __shared__ float s_part[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int co = blockIdx.x * 32 + lane;
    float s = 0.f;
    if (co < cout) {
#pragma unroll 8
        for (int c = warp; c < nchunk; c += 8) s += dbpart[(int64_t)c * cout + co];
    }
    s_part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && co < cout) {
        float t = 0.f;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += s_part[w][lane];
        db[co] = t;
    }
}

// wt[ci][tap][co] = w[co][26 - tap][ci]
__global__ void flip_transpose_kernel(const bf16* __restrict__ w, bf16* __restrict__ wt, int cin, int cout) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)27 * cin * cout) return;
    const int ci = (int)(e / (27 * cout));
    const int tap = (int)((e / cout) % 27);
    const int co = (int)(e % cout);
    wt[e] = w[((int64_t)co * 27 + (26 - tap)) * cin + ci];
}

__global__ void pool2_kernel(const bf16* __restrict__ in, bf16* __restrict__ out, uint8_t* __restrict__ arg, int N,
                             int D, int H, int W, int C) {
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * d * h * w * C;
    if (e >= total) return;
    const int c = (int)(e % C);
    const Vox P = decode(e / C, d, h, w);
    float best = -3.0e38f;
    int bi = 0;
    for (int k = 0; k < 8; ++k) {
        const int z = 2 * P.z + (k >> 2), y = 2 * P.y + ((k >> 1) & 1), x = 2 * P.x + (k & 1);
        const float val = __bfloat162float(in[((((int64_t)P.n * D + z) * H + y) * W + x) * C + c]);
        if (val > best) { best = val; bi = k; }
    }
    out[e] = __float2bfloat16_rn(best);
    arg[e] = (uint8_t)bi;
}

// g_in (full resolution) = scatter of g_out to the argmax child (+ g_in if accumulate).
__global__ void pool2_bwd_kernel(const bf16* __restrict__ gout, const uint8_t* __restrict__ arg,
                                 bf16* __restrict__ gin, const bf16* __restrict__ mask, int N, int D, int H, int W,
                                 int C, int accumulate) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * D * H * W * C;
    if (e >= total) return;
    const int c = (int)(e % C);
    const Vox P = decode(e / C, D, H, W);
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t o = ((((int64_t)P.n * d + P.z / 2) * h + P.y / 2) * w + P.x / 2) * C + c;
    const int k = ((P.z & 1) << 2) | ((P.y & 1) << 1) | (P.x & 1);
    float val = arg[o] == k ? __bfloat162float(gout[o]) : 0.f;
    if (accumulate) val += __bfloat162float(gin[e]);
    if (mask && !(__bfloat162float(mask[e]) > 0.f)) val = 0.f;
    gin[e] = __float2bfloat16_rn(val);
}

__global__ void upsample2_kernel(const bf16* __restrict__ in, bf16* __restrict__ out, int N, int d, int h, int w,
                                 int C) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * 8 * d * h * w * C;
    if (e >= total) return;
    const int c = (int)(e % C);
    const Vox P = decode(e / C, 2 * d, 2 * h, 2 * w);
    out[e] = in[((((int64_t)P.n * d + P.z / 2) * h + P.y / 2) * w + P.x / 2) * C + c];
}

__global__ void upsample2_bwd_kernel(const bf16* __restrict__ gout, bf16* __restrict__ gin,
                                     const bf16* __restrict__ mask, int N, int d, int h, int w, int C) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * d * h * w * C;
    if (e >= total) return;
    const int c = (int)(e % C);
    const Vox P = decode(e / C, d, h, w);
    float s = 0.f;
    for (int k = 0; k < 8; ++k) {
        const int z = 2 * P.z + (k >> 2), y = 2 * P.y + ((k >> 1) & 1), x = 2 * P.x + (k & 1);
        s += __bfloat162float(gout[((((int64_t)P.n * 2 * d + z) * 2 * h + y) * 2 * w + x) * C + c]);
    }
    if (mask && !(__bfloat162float(mask[e]) > 0.f)) s = 0.f;
    gin[e] = __float2bfloat16_rn(s);
}

__global__ void concat_kernel(const bf16* __restrict__ a, int ca, const bf16* __restrict__ b, int cb,
                              bf16* __restrict__ out, int64_t nvox) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = ca + cb;
    if (e >= nvox * C) return;
    const int64_t v = e / C;
    const int c = (int)(e % C);
    out[e] = c < ca ? a[v * ca + c] : b[v * cb + (c - ca)];
}

// ga = g[:, :ca]; gb (+)= g[:, ca:], then gb *= (mask_b > 0) when mask_b given.
__global__ void split_kernel(const bf16* __restrict__ g, int ca, int cb, bf16* __restrict__ ga, bf16* __restrict__ gb,
                             const bf16* __restrict__ mask_b, int accumulate_b, int64_t nvox) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = ca + cb;
    if (e >= nvox * C) return;
    const int64_t v = e / C;
    const int c = (int)(e % C);
    if (c < ca) {
        ga[v * ca + c] = g[e];
    } else {
        const int64_t o = v * cb + (c - ca);
        float val = __bfloat162float(g[e]);
        if (accumulate_b) val += __bfloat162float(gb[o]);
        if (mask_b && !(__bfloat162float(mask_b[o]) > 0.f)) val = 0.f;
        gb[o] = __float2bfloat16_rn(val);
    }
}

// Output head: y[v][o] = sum_c x[v][c] w[o][c] + b[o]  (FP32 out, cin <= 64, cout <= 8)
__global__ void head_fwd_kernel(const bf16* __restrict__ x, const float* __restrict__ w, const float* __restrict__ b,
                                float* __restrict__ y, int64_t nvox, int cin, int cout) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    float xs[64];
    for (int c = 0; c < cin; ++c) xs[c] = __bfloat162float(x[v * cin + c]);
    for (int o = 0; o < cout; ++o) {
        float s = b[o];
        for (int c = 0; c < cin; ++c) s = fmaf(xs[c], w[o * cin + c], s);
        y[v * cout + o] = s;
    }
}

// gx[v][c] = act'(d[v][c]) * sum_o gy[v][o] w[o][c]; d = the head's input x
// (ReLU) or its pre-activation (GELU)
__global__ void head_bwd_data_kernel(const float* __restrict__ gy, const float* __restrict__ w,
                                     const bf16* __restrict__ d, bf16* __restrict__ gx, int64_t nvox, int cin,
                                     int cout, int act) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    for (int c = 0; c < cin; ++c) {
        float s = 0.f;
        for (int o = 0; o < cout; ++o) s = fmaf(gy[v * cout + o], w[o * cin + c], s);
        gx[v * cin + c] = __float2bfloat16_rn(s * nn_act_grad(act, __bfloat162float(d[v * cin + c])));
    }
}

// g[e] *= act'(d[e]) in place
__global__ void act_bwd_kernel(bf16* __restrict__ g, const bf16* __restrict__ d, int64_t count, int act) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    g[e] = __float2bfloat16_rn(__bfloat162float(g[e]) * nn_act_grad(act, __bfloat162float(d[e])));
}

// Head weight/bias gradient partials per block: part[block][o*cin + c], part[block][cout*cin + o].
// ---- 16-byte (8-channel) forms of the memory kernels above, for channel counts that are
// multiples of 8: the same per-element arithmetic in the same order, one vector per thread.
union V8 {
    uint4 u;
    bf16 h[8];
};

// The vector forms need 16-byte aligned tensors (8-byte for the pool argmax); NULL passes.
__host__ inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
__host__ inline bool al8(const void* p) { return ((uintptr_t)p & 7u) == 0; }

__global__ void concat8_kernel(const uint4* __restrict__ a, int ca8, const uint4* __restrict__ b, int cb8,
                               uint4* __restrict__ out, int64_t nvox) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int C8 = ca8 + cb8;
    if (e >= nvox * C8) return;
    const int64_t v = e / C8;
    const int c = (int)(e - v * C8);
    out[e] = c < ca8 ? a[v * ca8 + c] : b[v * cb8 + (c - ca8)];
}

__global__ void split8_kernel(const uint4* __restrict__ g, int ca8, int cb8, uint4* __restrict__ ga, uint4* __restrict__ gb,
                              const uint4* __restrict__ mask_b, int accumulate_b, int64_t nvox) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int C8 = ca8 + cb8;
    if (e >= nvox * C8) return;
    const int64_t v = e / C8;
    const int c = (int)(e - v * C8);
    if (c < ca8) {
        ga[v * ca8 + c] = g[e];
        return;
    }
    const int64_t o = v * cb8 + (c - ca8);
    V8 in, acc, m, r;
    in.u = g[e];
    if (accumulate_b) acc.u = gb[o];
    if (mask_b) m.u = mask_b[o];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        float val = __bfloat162float(in.h[q]);
        if (accumulate_b) val += __bfloat162float(acc.h[q]);
        if (mask_b && !(__bfloat162float(m.h[q]) > 0.f)) val = 0.f;
        r.h[q] = __float2bfloat16_rn(val);
    }
    gb[o] = r.u;
}

__global__ void upsample8_kernel(const uint4* __restrict__ in, uint4* __restrict__ out, int N, int d, int h, int w,
                                 int C8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * 8 * d * h * w * C8;
    if (e >= total) return;
    const int64_t vo = e / C8;
    const int c = (int)(e - vo * C8);
    const Vox P = decode(vo, 2 * d, 2 * h, 2 * w);
    out[e] = in[((((int64_t)P.n * d + P.z / 2) * h + P.y / 2) * w + P.x / 2) * C8 + c];
}

__global__ void upsample8_bwd_kernel(const uint4* __restrict__ gout, uint4* __restrict__ gin,
                                     const uint4* __restrict__ mask, int N, int d, int h, int w, int C8) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * d * h * w * C8;
    if (e >= total) return;
    const int64_t vi = e / C8;
    const int c = (int)(e - vi * C8);
    const Vox P = decode(vi, d, h, w);
    float s[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] = 0.f;
    for (int k = 0; k < 8; ++k) {
        const int z = 2 * P.z + (k >> 2), y = 2 * P.y + ((k >> 1) & 1), x = 2 * P.x + (k & 1);
        V8 g;
        g.u = gout[((((int64_t)P.n * 2 * d + z) * 2 * h + y) * 2 * w + x) * C8 + c];
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] += __bfloat162float(g.h[q]);
    }
    V8 m, r;
    if (mask) m.u = mask[e];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        float val = s[q];
        if (mask && !(__bfloat162float(m.h[q]) > 0.f)) val = 0.f;
        r.h[q] = __float2bfloat16_rn(val);
    }
    gin[e] = r.u;
}

__global__ void pool8_kernel(const uint4* __restrict__ in, uint4* __restrict__ out, uint2* __restrict__ arg, int N, int D,
                             int H, int W, int C8) {
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * d * h * w * C8;
    if (e >= total) return;
    const int64_t vo = e / C8;
    const int c = (int)(e - vo * C8);
    const Vox P = decode(vo, d, h, w);
    float best[8];
    int bi[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        best[q] = -3.0e38f;
        bi[q] = 0;
    }
    for (int k = 0; k < 8; ++k) {
        const int z = 2 * P.z + (k >> 2), y = 2 * P.y + ((k >> 1) & 1), x = 2 * P.x + (k & 1);
        V8 v;
        v.u = in[((((int64_t)P.n * D + z) * H + y) * W + x) * C8 + c];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float val = __bfloat162float(v.h[q]);
            if (val > best[q]) {
                best[q] = val;
                bi[q] = k;
            }
        }
    }
    V8 r;
    uint32_t a0 = 0, a1 = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        r.h[q] = __float2bfloat16_rn(best[q]);
        if (q < 4) a0 |= (uint32_t)bi[q] << (8 * q);
        else a1 |= (uint32_t)bi[q] << (8 * (q - 4));
    }
    out[e] = r.u;
    arg[e] = make_uint2(a0, a1);
}

__global__ void pool8_bwd_kernel(const uint4* __restrict__ gout, const uint2* __restrict__ arg, uint4* __restrict__ gin,
                                 const uint4* __restrict__ mask, int N, int D, int H, int W, int C8, int accumulate) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)N * D * H * W * C8;
    if (e >= total) return;
    const int64_t vi = e / C8;
    const int c = (int)(e - vi * C8);
    const Vox P = decode(vi, D, H, W);
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t o = ((((int64_t)P.n * d + P.z / 2) * h + P.y / 2) * w + P.x / 2) * C8 + c;
    const int k = ((P.z & 1) << 2) | ((P.y & 1) << 1) | (P.x & 1);
    const uint2 a = arg[o];
    V8 g, acc, m, r;
    g.u = gout[o];
    if (accumulate) acc.u = gin[e];
    if (mask) m.u = mask[e];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int aq = (int)(((q < 4 ? a.x : a.y) >> (8 * (q & 3))) & 0xFFu);
        float val = aq == k ? __bfloat162float(g.h[q]) : 0.f;
        if (accumulate) val += __bfloat162float(acc.h[q]);
        if (mask && !(__bfloat162float(m.h[q]) > 0.f)) val = 0.f;
        r.h[q] = __float2bfloat16_rn(val);
    }
    gin[e] = r.u;
}

// Head weight gradient for the network's 1x1 head (16 -> 4) in one pass: each thread
// accumulates all 68 sums over a grid-stride set of voxels, then a fixed tree (warp
// shuffles, then the 8 warps in order) gives the block's partial.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) head_wgrad1_kernel(const float* __restrict__ gy, const bf16* __restrict__ x,
                                                         float* __restrict__ part, int64_t nvox) {
    constexpr int NOUT = COUT * CIN + COUT;
    __shared__ float sh[8][NOUT];
    float acc[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; ++k) acc[k] = 0.f;
    for (int64_t v = (int64_t)blockIdx.x * 256 + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * 256) {
        float g[COUT], xv[CIN];
#pragma unroll
        for (int o = 0; o < COUT; ++o) g[o] = gy[v * COUT + o];
#pragma unroll
        for (int c8 = 0; c8 < CIN / 8; ++c8) {
            V8 t;
            t.u = reinterpret_cast<const uint4*>(x + v * CIN)[c8];
#pragma unroll
            for (int q = 0; q < 8; ++q) xv[c8 * 8 + q] = __bfloat162float(t.h[q]);
        }
#pragma unroll
        for (int o = 0; o < COUT; ++o) {
#pragma unroll
            for (int c = 0; c < CIN; ++c) acc[o * CIN + c] += g[o] * xv[c];
            acc[COUT * CIN + o] += g[o];
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NOUT; ++k) {
        float t = acc[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (lane == 0) sh[warp][k] = t;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < NOUT; k += 256) {
        float t = 0.f;
#pragma unroll
        for (int w8 = 0; w8 < 8; ++w8) t += sh[w8][k];
        part[(int64_t)blockIdx.x * NOUT + k] = t;
    }
}

__global__ void __launch_bounds__(256) head_wgrad_kernel(const float* __restrict__ gy, const bf16* __restrict__ x,
                                                         float* __restrict__ part, int64_t nvox, int cin, int cout) {
    __shared__ float sh[256];
    const int nout = cout * cin + cout;
    for (int k = 0; k < nout; ++k) {
        const int o = k < cout * cin ? k / cin : k - cout * cin;
        const int c = k < cout * cin ? k % cin : -1;
        float s = 0.f;
        for (int64_t v = (int64_t)blockIdx.x * 256 + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * 256)
            s += gy[v * cout + o] * (c >= 0 ? __bfloat162float(x[v * cin + c]) : 1.f);
        sh[threadIdx.x] = s;
        __syncthreads();
        for (int off = 128; off > 0; off >>= 1) {
            if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(int64_t)blockIdx.x * nout + k] = sh[0];
        __syncthreads();
    }
}

__global__ void sum_partials_kernel(const float* __restrict__ part, float* __restrict__ out, int nblk, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * n + k];
    out[k] = s;
}

// Masked MSE: loss partials and gy = 2 (y - t) / count on mask voxels.
__global__ void __launch_bounds__(256) mse_kernel(const float* __restrict__ y, const float* __restrict__ t,
                                                  const uint8_t* __restrict__ m, float* __restrict__ gy,
                                                  float* __restrict__ part, int64_t nvox, int c, float inv_count) {
    __shared__ float sh[256];
    float s = 0.f;
    for (int64_t v = (int64_t)blockIdx.x * 256 + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * 256)
        for (int k = 0; k < c; ++k) {
            const int64_t e = v * c + k;
            const float d = m[v] ? y[e] - t[e] : 0.f;
            s += d * d;
            gy[e] = 2.f * d * inv_count;
        }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0] * inv_count;
}

// Adam on FP32 master weights; optionally writes a BF16 copy.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ p16, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float g = gr[e] + wd * p[e];
    const float mm = b1 * m[e] + (1.f - b1) * g;
    const float vv = b2 * v[e] + (1.f - b2) * g * g;
    m[e] = mm;
    v[e] = vv;
    const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    p[e] -= upd;
    if (p16) p16[e] = __float2bfloat16_rn(p[e]);
}

int blocks(int64_t n, int t = 256) { return (int)((n + t - 1) / t); }

int check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return LBM_OK;
    return lbm_set_err(nullptr, LBM_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int64_t lbm_nn_wgrad_scratch_floats(int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout) {
    const int64_t chunks = std::max(std::max(nn_wgrad_tc_chunks((int64_t)n * d * h * w), nn_wgrad_tma_chunks(n, d, h, w)),
                                    nn_wgrad_ws_chunks(n, d, h, w));
    return chunks * (27 * (int64_t)cin * cout + cout);
}

int lbm_nn_conv3d_wgrad(const void* in, const void* g, float* dw, float* db, float* scratch, int64_t scratch_floats,
                        int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout, void* stream) {
    const int64_t nvox = (int64_t)n * d * h * w;
    if (!in || !g || !dw || !scratch || nvox <= 0) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: bad arguments");
    if (scratch_floats < lbm_nn_wgrad_scratch_floats(n, d, h, w, cin, cout))
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: scratch too small");
    cudaStream_t s = (cudaStream_t)stream;
    const bool ws = nn_wgrad_ws_usable(cin, cout);
    const bool tma = !ws && nn_wgrad_tma_usable(cin, cout);
    const int nchunk = (int)(ws ? nn_wgrad_ws_chunks(n, d, h, w)
                                : (tma ? nn_wgrad_tma_chunks(n, d, h, w) : nn_wgrad_tc_chunks(nvox)));
    float* dbpart = scratch + (int64_t)nchunk * 27 * cin * cout;
    int rc = ws    ? nn_wgrad_ws(in, g, scratch, dbpart, n, d, h, w, cin, cout, s)
             : tma ? nn_wgrad_tma(in, g, scratch, dbpart, n, d, h, w, cin, cout, s)
                   : nn_wgrad_tc_launch(in, g, scratch, dbpart, n, d, h, w, cin, cout, s);
    if (rc) return rc;
    wgrad_reduce_kernel<<<(unsigned)(((int64_t)27 * cin * cout + 31) / 32), 256, 0, s>>>(scratch, dw, nchunk, cin, cout);
    rc = check("wgrad_reduce_kernel");
    if (rc || !db) return rc;
    bias_reduce_kernel<<<(unsigned)((cout + 31) / 32), 256, 0, s>>>(dbpart, db, nchunk, cout);
    return check("bias_reduce_kernel");
}

int lbm_nn_flip_transpose(const void* w, void* wt, int32_t cin, int32_t cout, void* stream) {
    flip_transpose_kernel<<<blocks((int64_t)27 * cin * cout), 256, 0, (cudaStream_t)stream>>>((const bf16*)w, (bf16*)wt,
                                                                                                cin, cout);
    return check("flip_transpose_kernel");
}

int lbm_nn_pool2(const void* in, void* out, uint8_t* arg, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                 void* stream) {
    if ((d | h | w) & 1) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_pool2: even sizes required");
    if (c % 8 == 0 && al16(in) && al16(out) && al8(arg)) {
        pool8_kernel<<<blocks((int64_t)n * (d / 2) * (h / 2) * (w / 2) * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)in, (uint4*)out, (uint2*)arg, n, d, h, w, c / 8);
        return check("pool8_kernel");
    }
    pool2_kernel<<<blocks((int64_t)n * (d / 2) * (h / 2) * (w / 2) * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)in, (bf16*)out, arg, n, d, h, w, c);
    return check("pool2_kernel");
}

int lbm_nn_pool2_bwd(const void* gout, const uint8_t* arg, void* gin, const void* mask, int32_t n, int32_t d,
                     int32_t h, int32_t w, int32_t c, int32_t accumulate, void* stream) {
    if (c % 8 == 0 && al16(gout) && al8(arg) && al16(gin) && al16(mask)) {
        pool8_bwd_kernel<<<blocks((int64_t)n * d * h * w * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)gout, (const uint2*)arg, (uint4*)gin, (const uint4*)mask, n, d, h, w, c / 8, accumulate);
        return check("pool8_bwd_kernel");
    }
    pool2_bwd_kernel<<<blocks((int64_t)n * d * h * w * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)gout, arg, (bf16*)gin, (const bf16*)mask, n, d, h, w, c, accumulate);
    return check("pool2_bwd_kernel");
}

int lbm_nn_upsample2(const void* in, void* out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void* stream) {
    if (c % 8 == 0 && al16(in) && al16(out)) {
        upsample8_kernel<<<blocks((int64_t)n * 8 * d * h * w * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)in, (uint4*)out, n, d, h, w, c / 8);
        return check("upsample8_kernel");
    }
    upsample2_kernel<<<blocks((int64_t)n * 8 * d * h * w * c), 256, 0, (cudaStream_t)stream>>>((const bf16*)in,
                                                                                                (bf16*)out, n, d, h, w, c);
    return check("upsample2_kernel");
}

int lbm_nn_upsample2_bwd(const void* gout, void* gin, const void* mask, int32_t n, int32_t d, int32_t h, int32_t w,
                         int32_t c, void* stream) {
    if (c % 8 == 0 && al16(gout) && al16(gin) && al16(mask)) {
        upsample8_bwd_kernel<<<blocks((int64_t)n * d * h * w * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)gout, (uint4*)gin, (const uint4*)mask, n, d, h, w, c / 8);
        return check("upsample8_bwd_kernel");
    }
    upsample2_bwd_kernel<<<blocks((int64_t)n * d * h * w * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)gout, (bf16*)gin, (const bf16*)mask, n, d, h, w, c);
    return check("upsample2_bwd_kernel");
}

int lbm_nn_concat(const void* a, int32_t ca, const void* b, int32_t cb, void* out, int64_t nvox, void* stream) {
    if (ca % 8 == 0 && cb % 8 == 0 && al16(a) && al16(b) && al16(out)) {
        concat8_kernel<<<blocks(nvox * ((ca + cb) / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)a, ca / 8, (const uint4*)b, cb / 8, (uint4*)out, nvox);
        return check("concat8_kernel");
    }
    concat_kernel<<<blocks(nvox * (ca + cb)), 256, 0, (cudaStream_t)stream>>>((const bf16*)a, ca, (const bf16*)b, cb,
                                                                              (bf16*)out, nvox);
    return check("concat_kernel");
}

int lbm_nn_split(const void* g, int32_t ca, int32_t cb, void* ga, void* gb, const void* mask_b, int32_t accumulate_b,
                 int64_t nvox, void* stream) {
    if (ca % 8 == 0 && cb % 8 == 0 && al16(g) && al16(ga) && al16(gb) && al16(mask_b)) {
        split8_kernel<<<blocks(nvox * ((ca + cb) / 8)), 256, 0, (cudaStream_t)stream>>>(
            (const uint4*)g, ca / 8, cb / 8, (uint4*)ga, (uint4*)gb, (const uint4*)mask_b, accumulate_b, nvox);
        return check("split8_kernel");
    }
    split_kernel<<<blocks(nvox * (ca + cb)), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)g, ca, cb, (bf16*)ga, (bf16*)gb, (const bf16*)mask_b, accumulate_b, nvox);
    return check("split_kernel");
}

int lbm_nn_head(const void* x, const float* w, const float* b, float* y, int64_t nvox, int32_t cin, int32_t cout,
                void* stream) {
    if (cin > 64 || cout > 8) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_head: cin <= 64, cout <= 8");
    head_fwd_kernel<<<blocks(nvox, 128), 128, 0, (cudaStream_t)stream>>>((const bf16*)x, w, b, y, nvox, cin, cout);
    return check("head_fwd_kernel");
}

int lbm_nn_head_bwd(const float* gy, const float* w, const void* x, void* gx, float* dw_db, float* scratch,
                    int64_t nvox, int32_t cin, int32_t cout, void* stream) {
    return lbm_nn_head_bwd_act(gy, w, x, nullptr, gx, dw_db, scratch, nvox, cin, cout, LBM_NN_ACT_RELU, stream);
}

int lbm_nn_head_bwd_act(const float* gy, const float* w, const void* x, const void* pre, void* gx, float* dw_db,
                        float* scratch, int64_t nvox, int32_t cin, int32_t cout, int32_t act, void* stream) {
    if (act != LBM_NN_ACT_RELU && act != LBM_NN_ACT_GELU)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_head_bwd_act: act 0 (ReLU) or 1 (GELU)");
    if (act == LBM_NN_ACT_GELU && !pre) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_head_bwd_act: GELU needs pre");
    cudaStream_t s = (cudaStream_t)stream;
    const bf16* d = (const bf16*)(act == LBM_NN_ACT_GELU ? pre : x);
    head_bwd_data_kernel<<<blocks(nvox, 128), 128, 0, s>>>(gy, w, d, (bf16*)gx, nvox, cin, cout, act);
    int rc = check("head_bwd_data_kernel");
    if (rc) return rc;
    const int nb = 256, nout = cout * cin + cout;
    if (cin == 16 && cout == 4 && al16(x))
        head_wgrad1_kernel<16, 4><<<nb, 256, 0, s>>>(gy, (const bf16*)x, scratch, nvox);
    else
        head_wgrad_kernel<<<nb, 256, 0, s>>>(gy, (const bf16*)x, scratch, nvox, cin, cout);
    rc = check("head_wgrad_kernel");
    if (rc) return rc;
    sum_partials_kernel<<<blocks(nout), 256, 0, s>>>(scratch, dw_db, nb, nout);
    return check("sum_partials_kernel");
}

int lbm_nn_act_bwd(void* g, const void* d, int64_t count, int32_t act, void* stream) {
    if (act != LBM_NN_ACT_RELU && act != LBM_NN_ACT_GELU)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_act_bwd: act 0 (ReLU) or 1 (GELU)");
    if (!g || !d || count < 0) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_act_bwd: null pointer or count < 0");
    if (count == 0) return LBM_OK;
    act_bwd_kernel<<<blocks(count, 256), 256, 0, (cudaStream_t)stream>>>((bf16*)g, (const bf16*)d, count, act);
    return check("act_bwd_kernel");
}

int lbm_nn_mse(const float* y, const float* t, const uint8_t* mask, float* gy, float* loss, float* scratch,
               int64_t nvox, int32_t c, float inv_count, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = 256;
    mse_kernel<<<nb, 256, 0, s>>>(y, t, mask, gy, scratch, nvox, c, inv_count);
    int rc = check("mse_kernel");
    if (rc) return rc;
    sum_partials_kernel<<<1, 256, 0, s>>>(scratch, loss, nb, 1);
    return check("sum_partials_kernel");
}

int lbm_nn_adam(float* p, const float* g, float* m, float* v, void* p16, int64_t n, float lr, float b1, float b2,
                float eps, int32_t step, float weight_decay, void* stream) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, (bf16*)p16, n, lr, b1, b2, eps, c1, c2,
                                                             weight_decay);
    return check("adam_kernel");
}

}  // extern "C"
