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
#include "nn_act.cuh"

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

// Wait for the phase with the given parity to complete; false after `limit` cycles (~1 s).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = TC_WAIT_CYCLES) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > limit) return false;
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

// MODE 0: out = relu(conv + bias); 1: out = conv * (mask > 0) (mask may be
// NULL); 2: pre = conv + bias, out = gelu(pre); 3: out = conv * gelu'(mask)
// (mask = the pre-activation; NULL: no factor).
template <int COUT, int MODE>
__global__ void __launch_bounds__(TC_THREADS) conv3d_tc_kernel(const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                              const float* __restrict__ bias,
                                                              const bf16* __restrict__ mask, bf16* __restrict__ out,
                                                              bf16* __restrict__ pre, int N, int D, int H, int W,
                                                              int cin) {
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
    // L1, where the 27 taps of neighbouring voxels find them again.  Per-thread
    // invariants (operand offsets, the voxel's row pointer, which of the three
    // shifts per axis stay inside the volume) are computed once.
    const bf16* vrow = in + (live ? v : 0) * cin;
    const uint32_t zok = live ? (1u | 2u | 4u) & ~((z == 0 ? 1u : 0u) | (z == D - 1 ? 4u : 0u)) : 0u;
    const uint32_t yok = (1u | 2u | 4u) & ~((y == 0 ? 1u : 0u) | (y == H - 1 ? 4u : 0u));
    const uint32_t xok = (1u | 2u | 4u) & ~((x == 0 ? 1u : 0u) | (x == W - 1 ? 4u : 0u));
    const uint32_t a_off0 = canon(tid, 0), a_off1 = canon(tid, 1);
    int q_tap = 0, q_ks = 0;   // (tap, K step) of the next step to load; steps are loaded in order
    auto load_step = [&](int q, int s) {
        const int tap = q_tap;
        if (++q_ks == kc) { q_ks = 0; ++q_tap; }
        const uint32_t sa = smem0 + (uint32_t)s * stage_bytes;
        const uint32_t sb = sa + 4096u;
        const int tz = tap / 9, ty = (tap / 3) % 3, tx = tap % 3;   // shift + 1 per axis
        const bool in_range = (zok >> tz) & (yok >> ty) & (xok >> tx) & 1u;
        const int64_t shift = ((int64_t)((tz - 1) * H + (ty - 1)) * W + (tx - 1)) * cin;
        const bf16* src = in_range ? vrow + shift + (q - tap * kc) * 16 : in;
        cp_async16_ca(sa + a_off0, src, in_range);
        cp_async16_ca(sa + a_off1, src + 8, in_range);
        // w[co][tap][ci]: tap * cin + 16 ks = 16 q
#pragma unroll
        for (int e0 = 0; e0 < COUT * 2; e0 += TC_THREADS) {
            const int e = e0 + tid;
            if (COUT * 2 % TC_THREADS == 0 || e < COUT * 2)
                cp_async16_ca(sb + canon(e >> 1, e & 1), w + (int64_t)(e >> 1) * 27 * cin + (e & 1) * 8 + (int64_t)q * 16,
                              true);
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
                __align__(16) bf16 pa[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    float r = acc[q];
                    if constexpr (MODE == 0) {
                        r = fmaxf(r + (bias ? bias[c0 + q] : 0.f), 0.f);
                    } else if constexpr (MODE == 1) {
                        if (mask && !(__bfloat162float(mask[v * COUT + c0 + q]) > 0.f)) r = 0.f;
                    } else if constexpr (MODE == 2) {
                        r = r + (bias ? bias[c0 + q] : 0.f);
                        pa[q] = __float2bfloat16_rn(r);
                        r = nn_gelu(r);
                    } else {
                        if (mask) r = r * nn_gelu_grad(__bfloat162float(mask[v * COUT + c0 + q]));
                    }
                    o[q] = __float2bfloat16_rn(r);
                }
                uint4* dst = reinterpret_cast<uint4*>(out + v * COUT + c0);
                dst[0] = reinterpret_cast<const uint4*>(o)[0];
                dst[1] = reinterpret_cast<const uint4*>(o)[1];
                if constexpr (MODE == 2) {
                    uint4* dp = reinterpret_cast<uint4*>(pre + v * COUT + c0);
                    dp[0] = reinterpret_cast<const uint4*>(pa)[0];
                    dp[1] = reinterpret_cast<const uint4*>(pa)[1];
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

template <int COUT, int MODE>
int launch_tc(const bf16* in, const bf16* w, const float* bias, const bf16* mask, bf16* out, bf16* pre, int n, int d,
              int h, int wd, int cin, cudaStream_t s) {
    const size_t smem = (size_t)TC_STAGES * (4096 + (size_t)COUT * 32);
    auto k = conv3d_tc_kernel<COUT, MODE>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d: shared memory attribute");
    const int64_t nvox = (int64_t)n * d * h * wd;
    const int grid = (int)((nvox + TC_M - 1) / TC_M);
    k<<<grid, TC_THREADS, smem, s>>>(in, w, bias, mask, out, pre, n, d, h, wd, cin);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_tc_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

// Self-test of the timeout path: one CTA allocates tensor memory, waits on an
// mbarrier whose phase nothing completes (no arrival is ever made) with a
// short bound, records the timeout in the error flag exactly as the
// convolution kernels do, frees its tensor memory and returns.
__global__ void __launch_bounds__(32) tc_timeout_selftest_kernel(long long limit) {
    __shared__ uint64_t s_bar;
    __shared__ uint32_t s_taddr;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_taddr)), "r"(32)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;
    const bool done = mbar_wait(&s_bar, 0, limit);
    if (!done && threadIdx.x == 0) atomicExch(&g_tc_error, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(32) : "memory");
}

// ---------------------------------------------------------------------------
// Weight gradient on the tensor cores.  For one tap and one chunk of
// WGT_CHUNK voxels, part[chunk][tap][co][ci] = sum_v g[v][co] * in[v + off][ci]
// is a GEMM with M = co (TMEM lanes, rows >= cout stay zero), N = ci (TMEM
// columns) and K = voxels.  g and in are channels-last, so each stage is
// written into the K-major operand layout with transposing 32-bit stores (two
// voxels x one channel each; see the work units below).  The global loads of
// the next stage are issued before the stores of the current one, and each
// unit's voxel coordinates advance incrementally instead of being divided out
// per stage.  Partials are summed over chunks in a
// fixed order by wgrad_reduce_kernel (nn_unet.cu).  The CTAs of the centre
// tap (no shift) also sum g over their chunk from the same loads: the bias
// gradient partials dbpart[chunk][co].
constexpr int WGT_CHUNK = 4096;
constexpr int WGT_KV = 64;                 // voxels per stage (four K = 16 MMAs)
constexpr int WGT_UA = 2, WGT_UB = 4;      // work units per thread and stage (cout <= 64, cin <= 128)

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
    // the 27 taps of one chunk are consecutive CTAs, so g and the input chunk are read from L2
    const int tap = blockIdx.x;
    const int64_t chunk = blockIdx.y;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t c0 = chunk * WGT_CHUNK;
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
    float dbacc[WGT_UA][8];
#pragma unroll
    for (int u = 0; u < WGT_UA; ++u)
#pragma unroll
        for (int h = 0; h < 8; ++h) dbacc[u][h] = 0.f;

    // Work units of a stage: (octet o of 8 voxels, 8-channel group c8, voxel pair p); a unit
    // loads 8 channels of voxels 8o + 2p and 8o + 2p + 1 and stores them as 8 32-bit words
    // (two K neighbours of one operand row).  Lanes 4g' + p of a warp rotate their 8 rows by
    // g', so the 32 lanes of one store hit 32 different banks.
    const int na = 4 * cout, nb = 4 * CIN;   // units per stage
    // B units follow the A units in thread order (B unit e on thread (e + na) mod 128), so
    // small layers spread over all 128 threads; lane bits 0-4 are unchanged (na % 32 == 0)
    const int boff = na & (TC_THREADS - 1);
    const int64_t vshift = ((int64_t)dz * H + dy) * W + dx;
    const int rot = (tid >> 2) & 7;
    uint4 ra[WGT_UA][2], rb[WGT_UB][2];
    // coordinates of each B unit's first voxel, advanced by WGT_KV voxels per stage
    int bx[WGT_UB], by[WGT_UB], bz[WGT_UB];
#pragma unroll
    for (int u = 0; u < WGT_UB; ++u) {
        const int e = ((tid - boff) & (TC_THREADS - 1)) + u * TC_THREADS, gq = e >> 2;
        int64_t v = c0 + (gq & 7) * 8 + 2 * (e & 3);
        bx[u] = (int)(v % W);
        v /= W;
        by[u] = (int)(v % H);
        bz[u] = (int)((v / H) % D);
    }
    auto inside = [&](int x, int y, int z) {
        return (unsigned)(x + dx) < (unsigned)W && (unsigned)(y + dy) < (unsigned)H && (unsigned)(z + dz) < (unsigned)D;
    };
    auto fetch = [&](int q) {   // stage q's global data into registers
        const int64_t s0 = c0 + (int64_t)q * WGT_KV;
        const int64_t lim = min(nvox, c0 + (int64_t)WGT_CHUNK);
#pragma unroll
        for (int u = 0; u < WGT_UA; ++u) {
            const int e = tid + u * TC_THREADS;
            ra[u][0] = ra[u][1] = make_uint4(0u, 0u, 0u, 0u);
            if (e < na) {
                const int gq = e >> 2, c8 = gq >> 3;
                const int64_t v = s0 + (gq & 7) * 8 + 2 * (e & 3);
                const bf16* src = g + v * cout + c8 * 8;
                if (v < lim) ra[u][0] = *reinterpret_cast<const uint4*>(src);
                if (v + 1 < lim) ra[u][1] = *reinterpret_cast<const uint4*>(src + cout);
            }
        }
#pragma unroll
        for (int u = 0; u < WGT_UB; ++u) {
            const int e = ((tid - boff) & (TC_THREADS - 1)) + u * TC_THREADS;
            rb[u][0] = rb[u][1] = make_uint4(0u, 0u, 0u, 0u);
            if (e < nb) {
                const int gq = e >> 2, c8 = gq >> 3;
                const int64_t v = s0 + (gq & 7) * 8 + 2 * (e & 3);
                int x1 = bx[u] + 1, y1 = by[u], z1 = bz[u];
                if (x1 == W) {
                    x1 = 0;
                    if (++y1 == H) {
                        y1 = 0;
                        if (++z1 == D) z1 = 0;
                    }
                }
                const bf16* src = in + (v + vshift) * CIN + c8 * 8;
                if (v < lim && inside(bx[u], by[u], bz[u])) rb[u][0] = *reinterpret_cast<const uint4*>(src);
                if (v + 1 < lim && inside(x1, y1, z1)) rb[u][1] = *reinterpret_cast<const uint4*>(src + CIN);
            }
            // advance to the next stage
            bx[u] += WGT_KV;
            while (bx[u] >= W) {
                bx[u] -= W;
                if (++by[u] == H) {
                    by[u] = 0;
                    if (++bz[u] == D) bz[u] = 0;
                }
            }
        }
    };
    // rotate the 8 BF16 elements of a 16-byte vector by `rot` positions: element h of the
    // result is element (h + rot) & 7 of the input
    auto rotate8 = [&](const uint4& a) {
        const int wq = rot >> 1;
        uint32_t w0 = a.x, w1 = a.y, w2 = a.z, w3 = a.w;
        uint32_t r0 = wq == 0 ? w0 : (wq == 1 ? w1 : (wq == 2 ? w2 : w3));
        uint32_t r1 = wq == 0 ? w1 : (wq == 1 ? w2 : (wq == 2 ? w3 : w0));
        uint32_t r2 = wq == 0 ? w2 : (wq == 1 ? w3 : (wq == 2 ? w0 : w1));
        uint32_t r3 = wq == 0 ? w3 : (wq == 1 ? w0 : (wq == 2 ? w1 : w2));
        if (rot & 1) {
            const uint32_t t0 = __funnelshift_r(r0, r1, 16), t1 = __funnelshift_r(r1, r2, 16);
            const uint32_t t2 = __funnelshift_r(r2, r3, 16), t3 = __funnelshift_r(r3, r0, 16);
            r0 = t0; r1 = t1; r2 = t2; r3 = t3;
        }
        return make_uint4(r0, r1, r2, r3);
    };
    // store a unit: rows c8*8 + ((hh + rot) & 7), K positions j0 and j0 + 1 of the stage
    auto put = [&](uint32_t base, uint32_t step_bytes, int e, const uint4& va, const uint4& vb) {
        const int gq = e >> 2, c8 = gq >> 3, j0 = (gq & 7) * 8 + 2 * (e & 3);
        const uint32_t sub = base + (uint32_t)(j0 >> 4) * step_bytes + (uint32_t)c8 * 256u +
                             (uint32_t)(((j0 & 15) >> 3) * 128 + (j0 & 7) * 2);
        const uint4 a = rotate8(va), b = rotate8(vb);
        const uint32_t wa[4] = {a.x, a.y, a.z, a.w}, wb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int hh = 0; hh < 8; ++hh) {
            const uint32_t lo = (wa[hh >> 1] >> ((hh & 1) * 16)) & 0xFFFFu;
            const uint32_t hi = (wb[hh >> 1] >> ((hh & 1) * 16)) & 0xFFFFu;
            const uint32_t addr = sub + (uint32_t)(((hh + rot) & 7) * 16);
            asm volatile("st.shared.u32 [%0], %1;" ::"r"(addr), "r"(lo | (hi << 16)) : "memory");
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
        for (int u = 0; u < WGT_UA; ++u) {
            const int e = tid + u * TC_THREADS;
            if (e < na) {
                put(sa, A_STEP, e, ra[u][0], ra[u][1]);
                if (centre) {
#pragma unroll
                    for (int h = 0; h < 8; ++h) {
                        const uint32_t w0 = (h >> 1) == 0 ? ra[u][0].x : ((h >> 1) == 1 ? ra[u][0].y : ((h >> 1) == 2 ? ra[u][0].z : ra[u][0].w));
                        const uint32_t w1 = (h >> 1) == 0 ? ra[u][1].x : ((h >> 1) == 1 ? ra[u][1].y : ((h >> 1) == 2 ? ra[u][1].z : ra[u][1].w));
                        dbacc[u][h] += __uint_as_float((w0 >> ((h & 1) * 16)) << 16) +
                                       __uint_as_float((w1 >> ((h & 1) * 16)) << 16);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < WGT_UB; ++u) {
            const int e = ((tid - boff) & (TC_THREADS - 1)) + u * TC_THREADS;
            if (e < nb) put(sb, B_STEP, e, rb[u][0], rb[u][1]);
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
        for (int slot = 0; slot < 32; ++slot) {   // (octet, pair) = (slot >> 2, slot & 3)
#pragma unroll
            for (int u = 0; u < WGT_UA; ++u) {
                const int e = tid + u * TC_THREADS;
                if (e < na && (((e >> 2) & 7) << 2 | (e & 3)) == slot)
#pragma unroll
                    for (int h = 0; h < 8; ++h) s_db[(e >> 5) * 8 + h] += dbacc[u][h];
            }
            __syncthreads();
        }
        if (tid < cout) dbpart[chunk * cout + tid] = s_db[tid];
    }
    if (!mbar_wait(&s_bar[2], 0)) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        if (warp * 32 < cout) {
            const int co = warp * 32 + (tid & 31);
            float* dst = part + ((chunk * 27 + tap) * cout + co) * CIN;
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

int lbm_nn_conv3d_act(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre,
                      int32_t n, int32_t d, int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode,
                      void* stream) {
    const int64_t nvox = (int64_t)n * d * h * wd;
    if (!in || !w || !out || nvox <= 0 || cin % 16 || cin <= 0 || cin > 128 || mode < 0 || mode > 3)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: cin must be a multiple of 16 in [16, 128]; mode 0..3");
    if (mode == 2 && !pre) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_act: mode 2 needs pre");
    cudaStream_t s = (cudaStream_t)stream;
    if (nn_halo_usable(cin, cout)) return nn_conv3d_halo(in, w, bias, mask, out, pre, n, d, h, wd, cin, cout, mode, s);
    if (nn_tma_usable(cin, cout)) return nn_conv3d_tma(in, w, bias, mask, out, pre, n, d, h, wd, cin, cout, mode, s);
    const bf16* I = (const bf16*)in;
    const bf16* Wt = (const bf16*)w;
    const bf16* M = (const bf16*)mask;
    bf16* O = (bf16*)out;
    bf16* P = (bf16*)pre;
#define LBM_TC(C)                                                                  \
    case C:                                                                        \
        switch (mode) {                                                            \
        case 0: return launch_tc<C, 0>(I, Wt, bias, M, O, P, n, d, h, wd, cin, s); \
        case 1: return launch_tc<C, 1>(I, Wt, bias, M, O, P, n, d, h, wd, cin, s); \
        case 2: return launch_tc<C, 2>(I, Wt, bias, M, O, P, n, d, h, wd, cin, s); \
        default: return launch_tc<C, 3>(I, Wt, bias, M, O, P, n, d, h, wd, cin, s); \
        }
    switch (cout) {
        LBM_TC(16) LBM_TC(32) LBM_TC(48) LBM_TC(64) LBM_TC(96)
    default:
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: cout must be 16, 32, 48, 64 or 96");
    }
#undef LBM_TC
}

int lbm_nn_conv3d(const void* in, const void* w, const float* bias, const void* mask, void* out, int32_t n, int32_t d,
                  int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode, void* stream) {
    if (mode != 0 && mode != 1) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d: mode 0 or 1");
    return lbm_nn_conv3d_act(in, w, bias, mask, out, nullptr, n, d, h, wd, cin, cout, mode, stream);
}

// Runs the timeout self-test (about 1e6 cycles of waiting on a barrier nothing
// completes) and waits for it; the flag it sets is read with lbm_nn_tc_status.
int lbm_nn_tc_timeout_selftest(void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    tc_timeout_selftest_kernel<<<1, 32, 0, s>>>(1000000LL);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("tc_timeout_selftest: ") + cudaGetErrorString(e));
    return LBM_OK;
}

// 0 when no tensor-core convolution has timed out since the last call; clears the flag.
int lbm_nn_tc_status(int32_t* timed_out) {
    if (!timed_out) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_tc_status: NULL");
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_tc_status: symbol copy failed");
    int vt = 0;
    if (nn_tma_take_error(&vt) != LBM_OK) return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_tc_status: symbol copy failed");
    *timed_out = v | vt;
    return LBM_OK;
}

}  // extern "C"

// Tensor-core weight-gradient partials (see conv3d_wgrad_tc_kernel); grid (27 taps, chunks).
int nn_wgrad_tc_launch(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int w, int cin,
                       int cout, cudaStream_t s) {
    if (cin % 16 || cin < 16 || cin > 128 || cout % 8 || cout < 8 || cout > 64)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: cin must be a multiple of 16 up to 128, cout a multiple of 8 up to 64");
    const int64_t nvox = (int64_t)n * d * h * w;
    if ((nvox + WGT_CHUNK - 1) / WGT_CHUNK > 65535)
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad: more than 65535 x 4096 voxels");
    const dim3 grid(27, (unsigned)((nvox + WGT_CHUNK - 1) / WGT_CHUNK));
    const size_t smem = 2 * (WGT_KV / 16) * (4096 + (size_t)cin * 32);
#define LBM_WG(C)                                                                                              \
    case C: {                                                                                                  \
        auto k = conv3d_wgrad_tc_kernel<C>;                                                                    \
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)    \
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad: shared memory attribute refused for " +  \
                                                       std::to_string(smem) + " bytes");                        \
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
