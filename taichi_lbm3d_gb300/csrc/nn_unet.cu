// Kernels of the warm-start network (a 3-level 3D U-Net, see unet.py):
// 3x3x3 convolutions, 2x max-pool, 2x nearest upsample, channel concat/split,
// 1x1 output head, masked MSE, Adam.  Activations are BF16, channels last
// (N, D, H, W, C); accumulation is FP32.
//
// conv3d_mma_kernel: implicit GEMM on the tensor cores (mma.sync m16n8k16
// BF16 -> FP32).  M = voxels (16 per warp), N = output channels, K = 27 taps x
// input channels; zero padding at the volume faces.  The same kernel computes
// the backward-data pass with the tap-flipped, transposed weights.  Epilogues:
// bias + ReLU (forward) or multiply by the ReLU mask of the layer input
// (backward).  conv3d_wgrad_kernel: weight gradient on the CUDA cores (FP32
// FMA, 4x4 register blocks), one partial per (voxel chunk, tap), summed in a
// fixed order by a second kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/lbm_nn.h"
#include "lbm_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

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

// MODE 0: out = relu(acc + bias); MODE 1: out = acc * (mask > 0) (mask may be NULL).
template <int NT, int MODE>
__global__ void __launch_bounds__(128) conv3d_mma_kernel(const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                         const float* __restrict__ bias,
                                                         const bf16* __restrict__ mask, bf16* __restrict__ out,
                                                         int N, int D, int H, int W, int cin) {
    constexpr int COUT = NT * 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t v0 = ((int64_t)blockIdx.x * 4 + warp) * 16;
    if (v0 >= nvox) return;
    const int g = lane >> 2, q = lane & 3;
    const int64_t va = v0 + g, vb = va + 8;
    const Vox A = decode(va, D, H, W), B = decode(vb, D, H, W);
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
    const int kc = cin >> 4;
    for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int za = A.z + dz, ya = A.y + dy, xa = A.x + dx;
        const int zb = B.z + dz, yb = B.y + dy, xb = B.x + dx;
        const bool ina = za >= 0 && za < D && ya >= 0 && ya < H && xa >= 0 && xa < W;
        const bool inb = zb >= 0 && zb < D && yb >= 0 && yb < H && xb >= 0 && xb < W;
        const bf16* pa = in + ((((int64_t)A.n * D + za) * H + ya) * W + xa) * cin + q * 2;
        const bf16* pb = in + ((((int64_t)B.n * D + zb) * H + yb) * W + xb) * cin + q * 2;
        const bf16* wt = w + (int64_t)tap * cin + q * 2;
        for (int c = 0; c < kc; ++c) {
            const uint32_t a0 = ina ? ld32(pa + c * 16) : 0u;
            const uint32_t a1 = inb ? ld32(pb + c * 16) : 0u;
            const uint32_t a2 = ina ? ld32(pa + c * 16 + 8) : 0u;
            const uint32_t a3 = inb ? ld32(pb + c * 16 + 8) : 0u;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const bf16* wp = wt + (int64_t)(t * 8 + g) * 27 * cin + c * 16;
                mma_bf16(acc[t], a0, a1, a2, a3, ld32(wp), ld32(wp + 8));
            }
        }
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int co = t * 8 + q * 2;
        float r0 = acc[t][0], r1 = acc[t][1], r2 = acc[t][2], r3 = acc[t][3];
        if constexpr (MODE == 0) {
            const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
            r0 = fmaxf(r0 + b0, 0.f);
            r1 = fmaxf(r1 + b1, 0.f);
            r2 = fmaxf(r2 + b0, 0.f);
            r3 = fmaxf(r3 + b1, 0.f);
        } else {
            if (mask) {
                const __nv_bfloat162 ma = *reinterpret_cast<const __nv_bfloat162*>(mask + va * COUT + co);
                const __nv_bfloat162 mb = *reinterpret_cast<const __nv_bfloat162*>(mask + vb * COUT + co);
                r0 = __bfloat162float(ma.x) > 0.f ? r0 : 0.f;
                r1 = __bfloat162float(ma.y) > 0.f ? r1 : 0.f;
                r2 = __bfloat162float(mb.x) > 0.f ? r2 : 0.f;
                r3 = __bfloat162float(mb.y) > 0.f ? r3 : 0.f;
            }
        }
        *reinterpret_cast<__nv_bfloat162*>(out + va * COUT + co) = __floats2bfloat162_rn(r0, r1);
        *reinterpret_cast<__nv_bfloat162*>(out + vb * COUT + co) = __floats2bfloat162_rn(r2, r3);
    }
}

// Weight gradient partials: part[chunk][tap][co][ci] = sum over the chunk's
// voxels v of g[v][co] * in[v + off(tap)][ci].
constexpr int WG_CHUNK = 4096, WG_SUB = 32;
__global__ void __launch_bounds__(256) conv3d_wgrad_kernel(const bf16* __restrict__ in, const bf16* __restrict__ g,
                                                           float* __restrict__ part, int N, int D, int H, int W,
                                                           int cin, int cout) {
    extern __shared__ float sm[];
    float* sg = sm;                       // [WG_SUB][cout]
    float* si = sm + WG_SUB * cout;       // [WG_SUB][cin]
    const int tap = blockIdx.y;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t c0 = (int64_t)blockIdx.x * WG_CHUNK;
    const int nco = cout / 4, nci = cin / 4;   // 4x4 blocks
    const int nblk = nco * nci;
    float acc[2][16];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[r][e] = 0.f;
    for (int64_t s0 = c0; s0 < c0 + WG_CHUNK && s0 < nvox; s0 += WG_SUB) {
        for (int e = threadIdx.x; e < WG_SUB * cout; e += blockDim.x) {
            const int64_t v = s0 + e / cout;
            sg[e] = v < nvox ? __bfloat162float(g[v * cout + e % cout]) : 0.f;
        }
        for (int e = threadIdx.x; e < WG_SUB * cin; e += blockDim.x) {
            const int64_t v = s0 + e / cin;
            float val = 0.f;
            if (v < nvox) {
                const Vox P = decode(v, D, H, W);
                const int z = P.z + dz, y = P.y + dy, x = P.x + dx;
                if (z >= 0 && z < D && y >= 0 && y < H && x >= 0 && x < W)
                    val = __bfloat162float(in[((((int64_t)P.n * D + z) * H + y) * W + x) * cin + e % cin]);
            }
            si[e] = val;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int b = threadIdx.x + r * blockDim.x;
            if (b < nblk) {
                const int bo = (b / nci) * 4, bi = (b % nci) * 4;
                for (int vv = 0; vv < WG_SUB; ++vv) {
                    float gg[4], ii[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        gg[u] = sg[vv * cout + bo + u];
                        ii[u] = si[vv * cin + bi + u];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int l = 0; l < 4; ++l) acc[r][u * 4 + l] = fmaf(gg[u], ii[l], acc[r][u * 4 + l]);
                }
            }
        }
        __syncthreads();
    }
    float* dst = part + ((int64_t)blockIdx.x * 27 + tap) * cout * cin;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int b = threadIdx.x + r * blockDim.x;
        if (b < nblk) {
            const int bo = (b / nci) * 4, bi = (b % nci) * 4;
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int l = 0; l < 4; ++l) dst[(bo + u) * cin + bi + l] = acc[r][u * 4 + l];
        }
    }
}

// dw[co][tap][ci] = sum over chunks (fixed order) of part[chunk][tap][co][ci].
__global__ void wgrad_reduce_kernel(const float* __restrict__ part, float* __restrict__ dw, int nchunk, int cin,
                                    int cout) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)27 * cout * cin;
    if (e >= total) return;
    const int tap = (int)(e / ((int64_t)cout * cin));
    const int co = (int)((e / cin) % cout), ci = (int)(e % cin);
    float s = 0.f;
    for (int c = 0; c < nchunk; ++c) s += part[((int64_t)c * 27 + tap) * cout * cin + (int64_t)co * cin + ci];
    dw[((int64_t)co * 27 + tap) * cin + ci] = s;
}

// db[co] = sum over voxels of g[v][co] (one block per channel, fixed order tree).
__global__ void __launch_bounds__(256) bias_grad_kernel(const bf16* __restrict__ g, float* __restrict__ db,
                                                        int64_t nvox, int cout) {
    __shared__ float sh[256];
    const int co = blockIdx.x;
    float s = 0.f;
    for (int64_t v = threadIdx.x; v < nvox; v += 256) s += __bfloat162float(g[v * cout + co]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[co] = sh[0];
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

// gx[v][c] = (x[v][c] > 0) * sum_o gy[v][o] w[o][c]
__global__ void head_bwd_data_kernel(const float* __restrict__ gy, const float* __restrict__ w,
                                     const bf16* __restrict__ x, bf16* __restrict__ gx, int64_t nvox, int cin,
                                     int cout) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    for (int c = 0; c < cin; ++c) {
        float s = 0.f;
        for (int o = 0; o < cout; ++o) s = fmaf(gy[v * cout + o], w[o * cin + c], s);
        gx[v * cin + c] = __float2bfloat16_rn(__bfloat162float(x[v * cin + c]) > 0.f ? s : 0.f);
    }
}

// Head weight/bias gradient partials per block: part[block][o*cin + c], part[block][cout*cin + o].
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

int lbm_nn_conv3d(const void* in, const void* w, const float* bias, const void* mask, void* out, int32_t n, int32_t d,
                  int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode, void* stream) {
    const int64_t nvox = (int64_t)n * d * h * wd;
    if (!in || !w || !out || nvox <= 0 || nvox % 16 || cin % 16 || cin <= 0 || (mode != 0 && mode != 1))
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: voxels and cin must be multiples of 16; mode 0 or 1");
    cudaStream_t s = (cudaStream_t)stream;
    const int grid = (int)((nvox / 16 + 3) / 4);
    const bf16* I = (const bf16*)in;
    const bf16* Wt = (const bf16*)w;
    const bf16* M = (const bf16*)mask;
    bf16* O = (bf16*)out;
#define LBM_CONV(NT)                                                                                  \
    case NT * 8:                                                                                      \
        if (mode == 0) conv3d_mma_kernel<NT, 0><<<grid, 128, 0, s>>>(I, Wt, bias, M, O, n, d, h, wd, cin); \
        else conv3d_mma_kernel<NT, 1><<<grid, 128, 0, s>>>(I, Wt, bias, M, O, n, d, h, wd, cin);          \
        break;
    switch (cout) {
        LBM_CONV(2) LBM_CONV(4) LBM_CONV(6) LBM_CONV(8) LBM_CONV(12)
    default:
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: cout must be 16, 32, 48, 64 or 96");
    }
#undef LBM_CONV
    return check("conv3d_mma_kernel");
}

int64_t lbm_nn_wgrad_scratch_floats(int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout) {
    const int64_t nvox = (int64_t)n * d * h * w;
    return ((nvox + WG_CHUNK - 1) / WG_CHUNK) * 27 * (int64_t)cin * cout;
}

int lbm_nn_conv3d_wgrad(const void* in, const void* g, float* dw, float* db, float* scratch, int64_t scratch_floats,
                        int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout, void* stream) {
    const int64_t nvox = (int64_t)n * d * h * w;
    if (!in || !g || !dw || !scratch || cin % 4 || cout % 4 || (cin / 4) * (cout / 4) > 512)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: bad arguments");
    if (scratch_floats < lbm_nn_wgrad_scratch_floats(n, d, h, w, cin, cout))
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: scratch too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int nchunk = (int)((nvox + WG_CHUNK - 1) / WG_CHUNK);
    const size_t smem = sizeof(float) * WG_SUB * (cin + cout);
    conv3d_wgrad_kernel<<<dim3(nchunk, 27), 256, smem, s>>>((const bf16*)in, (const bf16*)g, scratch, n, d, h, w, cin,
                                                          cout);
    int rc = check("conv3d_wgrad_kernel");
    if (rc) return rc;
    wgrad_reduce_kernel<<<blocks((int64_t)27 * cin * cout), 256, 0, s>>>(scratch, dw, nchunk, cin, cout);
    rc = check("wgrad_reduce_kernel");
    if (rc || !db) return rc;
    bias_grad_kernel<<<cout, 256, 0, s>>>((const bf16*)g, db, nvox, cout);
    return check("bias_grad_kernel");
}

int lbm_nn_flip_transpose(const void* w, void* wt, int32_t cin, int32_t cout, void* stream) {
    flip_transpose_kernel<<<blocks((int64_t)27 * cin * cout), 256, 0, (cudaStream_t)stream>>>((const bf16*)w, (bf16*)wt,
                                                                                                cin, cout);
    return check("flip_transpose_kernel");
}

int lbm_nn_pool2(const void* in, void* out, uint8_t* arg, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                 void* stream) {
    if ((d | h | w) & 1) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_pool2: even sizes required");
    pool2_kernel<<<blocks((int64_t)n * (d / 2) * (h / 2) * (w / 2) * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)in, (bf16*)out, arg, n, d, h, w, c);
    return check("pool2_kernel");
}

int lbm_nn_pool2_bwd(const void* gout, const uint8_t* arg, void* gin, const void* mask, int32_t n, int32_t d,
                     int32_t h, int32_t w, int32_t c, int32_t accumulate, void* stream) {
    pool2_bwd_kernel<<<blocks((int64_t)n * d * h * w * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)gout, arg, (bf16*)gin, (const bf16*)mask, n, d, h, w, c, accumulate);
    return check("pool2_bwd_kernel");
}

int lbm_nn_upsample2(const void* in, void* out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void* stream) {
    upsample2_kernel<<<blocks((int64_t)n * 8 * d * h * w * c), 256, 0, (cudaStream_t)stream>>>((const bf16*)in,
                                                                                                (bf16*)out, n, d, h, w, c);
    return check("upsample2_kernel");
}

int lbm_nn_upsample2_bwd(const void* gout, void* gin, const void* mask, int32_t n, int32_t d, int32_t h, int32_t w,
                         int32_t c, void* stream) {
    upsample2_bwd_kernel<<<blocks((int64_t)n * d * h * w * c), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)gout, (bf16*)gin, (const bf16*)mask, n, d, h, w, c);
    return check("upsample2_bwd_kernel");
}

int lbm_nn_concat(const void* a, int32_t ca, const void* b, int32_t cb, void* out, int64_t nvox, void* stream) {
    concat_kernel<<<blocks(nvox * (ca + cb)), 256, 0, (cudaStream_t)stream>>>((const bf16*)a, ca, (const bf16*)b, cb,
                                                                              (bf16*)out, nvox);
    return check("concat_kernel");
}

int lbm_nn_split(const void* g, int32_t ca, int32_t cb, void* ga, void* gb, const void* mask_b, int32_t accumulate_b,
                 int64_t nvox, void* stream) {
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
    cudaStream_t s = (cudaStream_t)stream;
    head_bwd_data_kernel<<<blocks(nvox, 128), 128, 0, s>>>(gy, w, (const bf16*)x, (bf16*)gx, nvox, cin, cout);
    int rc = check("head_bwd_data_kernel");
    if (rc) return rc;
    const int nb = 256, nout = cout * cin + cout;
    head_wgrad_kernel<<<nb, 256, 0, s>>>(gy, (const bf16*)x, scratch, nvox, cin, cout);
    rc = check("head_wgrad_kernel");
    if (rc) return rc;
    sum_partials_kernel<<<blocks(nout), 256, 0, s>>>(scratch, dw_db, nb, nout);
    return check("sum_partials_kernel");
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
