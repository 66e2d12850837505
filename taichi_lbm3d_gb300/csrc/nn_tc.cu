// 3x3x3 convolution of the warm-start network on the 5th-generation tensor
// cores: tcgen05.mma (BF16 x BF16 -> FP32) with the accumulator in tensor
// memory.  Implicit GEMM: M = 128 consecutive voxels per CTA (one TMEM lane
// each), N = output channels (16..96), K = 27 taps x input channels.
//
// Per K step of 16 channels of one tap (one pipeline stage): each of the 128
// threads gathers 32 bytes of its voxel's shifted input row (zero for taps
// outside the volume) with 16-byte cp.async copies into the canonical K-major
// layout of the MMA operand (8-row x 16-byte core matrices; LBO = 128 B between
// the two core matrices of the K step, SBO = 256 B between 8-row groups), and
// the weights of that step the same way; then one elected thread issues the
// K = 16 MMA and commits it to the stage's mbarrier.  Eight stages of 5-7 KB:
// the copies of the next six steps are in flight while the current one is
// multiplied, a stage is refilled two steps after its MMA was issued, and
// several CTAs share an SM.
// After the last tap the accumulator is read back with tcgen05.ld (warp w owns
// lanes 32w..32w+31), and the epilogue applies bias + ReLU (forward) or the
// ReLU mask of the layer input (backward data) and stores BF16.
//
// Every wait on an mbarrier is bounded (about a second of clock cycles); on a
// timeout the CTA records an error flag, waits (bounded) for its own MMAs,
// frees its tensor memory and exits.  lbm_nn_tc_status reads the flag.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm_nn.h"
#include "lbm_internal.h"

namespace {
typedef __nv_bfloat16 bf16;

constexpr int TC_M = 128;
constexpr int TC_THREADS = 128;
constexpr int TC_STAGES = 8;
constexpr int TC_AHEAD = 6;    // K steps whose copies are in flight ahead of the one multiplied
constexpr long long TC_WAIT_CYCLES = 2000000000LL;   // about 1 s at 2 GHz

__device__ int g_tc_error;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Wait for the phase with the given parity to complete; false after ~1 s.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    }
}

__device__ __forceinline__ void cp_async16_ca(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;   // fixed 0b001 at bits 46-48
    return d;                  // base offset 0, swizzle mode 0 (none)
}

// Instruction descriptor of kind::f16: FP32 accumulate, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
    return (1u << 4)                       // D: F32
           | (1u << 7)                     // A: BF16
           | (1u << 10)                    // B: BF16
           | ((uint32_t)(n >> 3) << 17)    // N / 8
           | ((uint32_t)(m >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void tc_mma(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Byte offset of (row, 8-element chunk h) of a K = 16 step in the canonical layout.
__device__ __forceinline__ uint32_t canon(int row, int h) { return (uint32_t)((row >> 3) * 256 + h * 128 + (row & 7) * 16); }

template <int COUT, int MODE>
__global__ void __launch_bounds__(TC_THREADS) conv3d_tc_kernel(const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                              const float* __restrict__ bias,
                                                              const bf16* __restrict__ mask, bf16* __restrict__ out,
                                                              int N, int D, int H, int W, int cin) {
    constexpr uint32_t NCOL = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);
    constexpr uint32_t IDESC = mma_idesc(TC_M, COUT);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t s_bar[TC_STAGES + 1];   // per-stage "consumed" + final "done"
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int kc = cin >> 4;                              // K steps of 16 channels per tap
    const uint32_t stage_bytes = 4096u + COUT * 32u;      // A: 128 rows x 32 B, B: COUT rows x 32 B
    const uint32_t smem0 = smem_u32(smem);

    if (tid == 0) {
        for (int s = 0; s <= TC_STAGES; ++s) mbar_init(&s_bar[s], 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_taddr)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;

    // this thread's output voxel (row of the tile)
    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t v = (int64_t)blockIdx.x * TC_M + tid;
    const bool live = v < nvox;
    int x = 0, y = 0, z = 0, n = 0;
    if (live) {
        x = (int)(v % W);
        int64_t t = v / W;
        y = (int)(t % H);
        t /= H;
        z = (int)(t % D);
        n = (int)(t / D);
    }

    // gather K step q (tap q / kc, channels 16 (q % kc) .. +15) into stage s:
    // A = this thread's shifted input row (zero outside the volume),
    // B = w[co][tap][ci] (row co, K = ci).  cp.async.ca keeps the input rows in
    // L1, where the 27 taps of neighbouring voxels find them again.
    auto load_step = [&](int q, int s) {
        const int tap = q / kc, ks = q - tap * kc;
        const uint32_t sa = smem0 + (uint32_t)s * stage_bytes;
        const uint32_t sb = sa + 4096u;
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int zz = z + dz, yy = y + dy, xx = x + dx;
        const bool in_range = live && zz >= 0 && zz < D && yy >= 0 && yy < H && xx >= 0 && xx < W;
        const bf16* src = in_range ? in + ((((int64_t)n * D + zz) * H + yy) * W + xx) * cin + ks * 16 : in;
        cp_async16_ca(sa + canon(tid, 0), src, in_range);
        cp_async16_ca(sa + canon(tid, 1), src + 8, in_range);
        for (int e = tid; e < COUT * 2; e += TC_THREADS) {
            const int co = e >> 1, h = e & 1;
            cp_async16_ca(sb + canon(co, h), w + ((int64_t)co * 27 + tap) * cin + ks * 16 + h * 8, true);
        }
    };

    // K steps run through TC_STAGES stages; the copies of the next TC_AHEAD
    // steps are in flight while the current one is multiplied, and a stage is
    // refilled TC_STAGES - TC_AHEAD steps after its MMA was issued, so that
    // MMA has normally finished by then.
    const int nq = 27 * kc;
#pragma unroll 1
    for (int q = 0; q < TC_AHEAD; ++q) {
        if (q < nq) load_step(q, q);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
#pragma unroll 1
    for (int q = 0; q < nq; ++q) {
        const int qn = q + TC_AHEAD;   // step to prefetch
        if (qn < nq) {
            const int sn = qn % TC_STAGES;
            if (qn >= TC_STAGES) {
                // the MMA of step qn - TC_STAGES, which read stage sn, has completed
                if (!mbar_wait(&s_bar[sn], (uint32_t)((qn / TC_STAGES - 1) & 1))) s_fail = 1;
                __syncthreads();
                if (s_fail) break;
            }
            load_step(qn, sn);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group %0;" ::"n"(TC_AHEAD) : "memory");   // step q's copies are complete
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            const int s = q % TC_STAGES;
            const uint32_t sa = smem0 + (uint32_t)s * stage_bytes;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            tc_mma(taddr, smem_desc(sa, 128, 256), smem_desc(sa + 4096u, 128, 256), IDESC, q > 0 ? 1u : 0u);
            tc_commit(&s_bar[s]);
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");   // no copies left in flight on any path
    // all MMAs issued so far complete -> "done"
    if (tid == 0) tc_commit(&s_bar[TC_STAGES]);
    const bool done = mbar_wait(&s_bar[TC_STAGES], 0);
    if (!done) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);   // this warp's 32 lanes
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tc_ld16(tw + (uint32_t)c0, acc);
            if (live) {
                __align__(16) bf16 o[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    float r = acc[q];
                    if constexpr (MODE == 0) {
                        r = fmaxf(r + (bias ? bias[c0 + q] : 0.f), 0.f);
                    } else {
                        if (mask && !(__bfloat162float(mask[v * COUT + c0 + q]) > 0.f)) r = 0.f;
                    }
                    o[q] = __float2bfloat16_rn(r);
                }
                uint4* dst = reinterpret_cast<uint4*>(out + v * COUT + c0);
                dst[0] = reinterpret_cast<const uint4*>(o)[0];
                dst[1] = reinterpret_cast<const uint4*>(o)[1];
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_tc_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(NCOL) : "memory");
}

template <int COUT, int MODE>
int launch_tc(const bf16* in, const bf16* w, const float* bias, const bf16* mask, bf16* out, int n, int d, int h,
              int wd, int cin, cudaStream_t s) {
    const size_t smem = (size_t)TC_STAGES * (4096 + (size_t)COUT * 32);
    auto k = conv3d_tc_kernel<COUT, MODE>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d: shared memory attribute");
    const int64_t nvox = (int64_t)n * d * h * wd;
    const int grid = (int)((nvox + TC_M - 1) / TC_M);
    k<<<grid, TC_THREADS, smem, s>>>(in, w, bias, mask, out, n, d, h, wd, cin);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_tc_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// Weight gradient on the tensor cores.  For one tap and one chunk of
// WGT_CHUNK voxels, part[chunk][tap][co][ci] = sum_v g[v][co] * in[v + off][ci]
// is a GEMM with M = co (TMEM lanes, rows >= cout stay zero), N = ci (TMEM
// columns) and K = voxels.  g and in are channels-last, so each stage is
// written into the K-major operand layout with a transposing store: a thread
// loads 8 channels of one voxel (16 bytes) and stores them as 8 two-byte
// elements of 8 operand rows.  The global loads of the next stage are issued
// before the stores of the current one.  Partials are summed over chunks in a
// fixed order by wgrad_reduce_kernel (nn_unet.cu).  The CTAs of the centre
// tap (no shift) also sum g over their chunk from the same loads: the bias
// gradient partials dbpart[chunk][co].
constexpr int WGT_CHUNK = 4096;
constexpr int WGT_KV = 64;                 // voxels per stage (four K = 16 MMAs)
constexpr int WGT_MAXA = 4, WGT_MAXB = 8;  // 16-byte loads per thread and stage (cout <= 64, cin <= 128)

template <int CIN>
__global__ void __launch_bounds__(TC_THREADS) conv3d_wgrad_tc_kernel(const bf16* __restrict__ in,
                                                                    const bf16* __restrict__ g,
                                                                    float* __restrict__ part,
                                                                    float* __restrict__ dbpart, int N, int D, int H,
                                                                    int W, int cout) {
    constexpr uint32_t NCOL = CIN <= 32 ? 32 : (CIN <= 64 ? 64 : 128);
    constexpr uint32_t IDESC = mma_idesc(TC_M, CIN);
    constexpr uint32_t A_STEP = 4096u;                 // 128 rows x 32 B per K = 16
    constexpr uint32_t B_STEP = (uint32_t)CIN * 32u;
    constexpr int KS = WGT_KV / 16;                    // MMAs per stage
    constexpr uint32_t STAGE = KS * (A_STEP + B_STEP);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t s_bar[3];
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;
    __shared__ float s_db[64];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int tap = blockIdx.y;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t c0 = (int64_t)blockIdx.x * WGT_CHUNK;
    const uint32_t smem0 = smem_u32(smem);

    // zero both stages once: A rows >= cout are never written
    for (uint32_t e = tid; e < 2 * STAGE / 16; e += TC_THREADS)
        reinterpret_cast<uint4*>(smem)[e] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&s_bar[b], 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < 64) s_db[tid] = 0.f;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_taddr)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;
    const bool centre = tap == 13;
    float dbacc[WGT_MAXA][8];
#pragma unroll
    for (int u = 0; u < WGT_MAXA; ++u)
#pragma unroll
        for (int h = 0; h < 8; ++h) dbacc[u][h] = 0.f;

    const int ga = WGT_KV * (cout / 8), gb = WGT_KV * (CIN / 8);   // (voxel, 8-channel group) pairs
    uint4 ra[WGT_MAXA], rb[WGT_MAXB];
    auto fetch = [&](int q) {   // stage q's global data into registers
        const int64_t s0 = c0 + (int64_t)q * WGT_KV;
#pragma unroll
        for (int u = 0; u < WGT_MAXA; ++u) {
            const int e = tid + u * TC_THREADS;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (e < ga) {
                const int j = e % WGT_KV, c8 = e / WGT_KV;
                const int64_t v = s0 + j;
                if (v < nvox && v < c0 + WGT_CHUNK) val = *reinterpret_cast<const uint4*>(g + v * cout + c8 * 8);
            }
            ra[u] = val;
        }
#pragma unroll
        for (int u = 0; u < WGT_MAXB; ++u) {
            const int e = tid + u * TC_THREADS;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (e < gb) {
                const int j = e % WGT_KV, c8 = e / WGT_KV;
                const int64_t v = s0 + j;
                if (v < nvox && v < c0 + WGT_CHUNK) {
                    int64_t t = v;
                    const int x = (int)(t % W) + dx;
                    t /= W;
                    const int y = (int)(t % H) + dy;
                    t /= H;
                    const int z = (int)(t % D) + dz;
                    const int nn = (int)(t / D);
                    if (z >= 0 && z < D && y >= 0 && y < H && x >= 0 && x < W)
                        val = *reinterpret_cast<const uint4*>(in + ((((int64_t)nn * D + z) * H + y) * W + x) * CIN + c8 * 8);
                }
            }
            rb[u] = val;
        }
    };
    // transposing store: element (row, k) of a K = 16 step at canon(row, k / 8) + (k % 8) * 2
    auto put = [&](uint32_t base, uint32_t step_bytes, int j, int c8, const uint4& val) {
        const uint32_t sub = base + (uint32_t)(j >> 4) * step_bytes;
        const int k = j & 15;
        const uint32_t off = (uint32_t)((k >> 3) * 128 + (k & 7) * 2);
        const uint32_t w4[4] = {val.x, val.y, val.z, val.w};
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            const int row = c8 * 8 + h;
            const uint16_t b16 = (uint16_t)(w4[h >> 1] >> ((h & 1) * 16));
            const uint32_t addr = sub + (uint32_t)((row >> 3) * 256 + (row & 7) * 16) + off;
            asm volatile("st.shared.u16 [%0], %1;" ::"r"(addr), "h"(b16) : "memory");
        }
    };

    const int nq = WGT_CHUNK / WGT_KV;
    fetch(0);
#pragma unroll 1
    for (int q = 0; q < nq; ++q) {
        const int s = q & 1;
        if (q >= 2) {   // the MMAs of step q - 2, which read stage s, have completed
            if (!mbar_wait(&s_bar[s], (uint32_t)((q / 2 - 1) & 1))) s_fail = 1;
            __syncthreads();
            if (s_fail) break;
        }
        const uint32_t sa = smem0 + (uint32_t)s * STAGE, sb = sa + KS * A_STEP;
#pragma unroll
        for (int u = 0; u < WGT_MAXA; ++u) {
            const int e = tid + u * TC_THREADS;
            if (e < ga) {
                put(sa, A_STEP, e % WGT_KV, e / WGT_KV, ra[u]);
                if (centre) {
                    const uint32_t w4[4] = {ra[u].x, ra[u].y, ra[u].z, ra[u].w};
#pragma unroll
                    for (int h = 0; h < 8; ++h)
                        dbacc[u][h] += __uint_as_float((w4[h >> 1] >> ((h & 1) * 16)) << 16);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < WGT_MAXB; ++u) {
            const int e = tid + u * TC_THREADS;
            if (e < gb) put(sb, B_STEP, e % WGT_KV, e / WGT_KV, rb[u]);
        }
        if (q + 1 < nq) fetch(q + 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int k2 = 0; k2 < KS; ++k2)
                tc_mma(taddr, smem_desc(sa + k2 * A_STEP, 128, 256), smem_desc(sb + k2 * B_STEP, 128, 256), IDESC,
                       (q > 0 || k2 > 0) ? 1u : 0u);
            tc_commit(&s_bar[s]);
        }
    }
    if (tid == 0) tc_commit(&s_bar[2]);
    if (centre) {   // bias-gradient partial of this chunk: fixed-order shared reduction
        for (int j0 = 0; j0 < WGT_KV; ++j0) {
#pragma unroll
            for (int u = 0; u < WGT_MAXA; ++u) {
                const int e = tid + u * TC_THREADS;
                if (e < ga && e % WGT_KV == j0)
#pragma unroll
                    for (int h = 0; h < 8; ++h) s_db[(e / WGT_KV) * 8 + h] += dbacc[u][h];
            }
            __syncthreads();
        }
        if (tid < cout) dbpart[(int64_t)blockIdx.x * cout + tid] = s_db[tid];
    }
    if (!mbar_wait(&s_bar[2], 0)) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        if (warp * 32 < cout) {
            const int co = warp * 32 + (tid & 31);
            float* dst = part + (((int64_t)blockIdx.x * 27 + tap) * cout + co) * CIN;
#pragma unroll
            for (int c = 0; c < CIN; c += 16) {
                float acc[16];
                tc_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc);
                if (co < cout) {
#pragma unroll
                    for (int q4 = 0; q4 < 4; ++q4)
                        reinterpret_cast<float4*>(dst + c)[q4] = make_float4(acc[4 * q4], acc[4 * q4 + 1], acc[4 * q4 + 2], acc[4 * q4 + 3]);
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_tc_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(NCOL) : "memory");
}
}  // namespace

extern "C" {

int lbm_nn_conv3d(const void* in, const void* w, const float* bias, const void* mask, void* out, int32_t n, int32_t d,
                  int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode, void* stream) {
    const int64_t nvox = (int64_t)n * d * h * wd;
    if (!in || !w || !out || nvox <= 0 || cin % 16 || cin <= 0 || cin > 128 || (mode != 0 && mode != 1))
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: cin must be a multiple of 16 in [16, 128]; mode 0 or 1");
    cudaStream_t s = (cudaStream_t)stream;
    const bf16* I = (const bf16*)in;
    const bf16* Wt = (const bf16*)w;
    const bf16* M = (const bf16*)mask;
    bf16* O = (bf16*)out;
#define LBM_TC(C)                                                                               \
    case C:                                                                                     \
        return mode == 0 ? launch_tc<C, 0>(I, Wt, bias, M, O, n, d, h, wd, cin, s)              \
                         : launch_tc<C, 1>(I, Wt, bias, M, O, n, d, h, wd, cin, s);
    switch (cout) {
        LBM_TC(16) LBM_TC(32) LBM_TC(48) LBM_TC(64) LBM_TC(96)
    default:
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: cout must be 16, 32, 48, 64 or 96");
    }
#undef LBM_TC
}

// 0 when no tensor-core convolution has timed out since the last call; clears the flag.
int lbm_nn_tc_status(int32_t* timed_out) {
    if (!timed_out) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_tc_status: NULL");
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_tc_status: symbol copy failed");
    *timed_out = v;
    return LBM_OK;
}

}  // extern "C"

// Tensor-core weight-gradient partials (see conv3d_wgrad_tc_kernel); grid (chunks, 27).
int nn_wgrad_tc_launch(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int w, int cin,
                       int cout, cudaStream_t s) {
    if (cin % 16 || cin < 16 || cin > 128 || cout % 8 || cout < 8 || cout > 64)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: cin must be a multiple of 16 up to 128, cout a multiple of 8 up to 64");
    const int64_t nvox = (int64_t)n * d * h * w;
    const dim3 grid((unsigned)((nvox + WGT_CHUNK - 1) / WGT_CHUNK), 27);
    const size_t smem = 2 * (WGT_KV / 16) * (4096 + (size_t)cin * 32);
#define LBM_WG(C)                                                                                              \
    case C: {                                                                                                  \
        auto k = conv3d_wgrad_tc_kernel<C>;                                                                    \
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)    \
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad: shared memory attribute");            \
        k<<<grid, TC_THREADS, smem, s>>>((const bf16*)in, (const bf16*)g, part, dbpart, n, d, h, w, cout);     \
        break;                                                                                                 \
    }
    switch (cin) {
        LBM_WG(16) LBM_WG(32) LBM_WG(48) LBM_WG(64) LBM_WG(80) LBM_WG(96) LBM_WG(112) LBM_WG(128)
    }
#undef LBM_WG
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_wgrad_tc_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}
int64_t nn_wgrad_tc_chunks(int64_t nvox) { return (nvox + WGT_CHUNK - 1) / WGT_CHUNK; }
