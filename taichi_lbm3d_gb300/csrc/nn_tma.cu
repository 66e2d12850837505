// 3x3x3 convolutions of the warm-start network on tcgen05.mma with operands
// moved by the tensor memory accelerator (TMA) or from a shared-memory halo.
// Four kernels, chosen per layer shape by lbm_nn_conv3d_act /
// lbm_nn_conv3d_wgrad (nn_tc.cu, nn_unet.cu):
//   conv3d_tma_kernel        forward / backward-data, im2col TMA loads per tap
//   conv3d_halo_kernel       forward / backward-data of narrow layers, one halo
//                            and all weights per CTA, taps as descriptor offsets
//   conv3d_wgrad_tma_kernel  weight gradient from tiled TMA boxes (MN-major)
//   conv3d_wgrad_ws_kernel   weight gradient, warp-specialised: one halo box per
//                            block, copy warps build the tap slots
// Each kernel's own comment describes its layout.  The first:
//
// Implicit GEMM as in nn_tc.cu (M = 128 consecutive voxels per CTA, one TMEM
// lane each; N = output channels; K = 27 taps x input channels), but a
// pipeline stage holds a whole tap and nothing is gathered by the threads:
//  * A: one im2col TMA load per channel part brings, for the tap's offsets
//    (tx, ty, tz), the input rows of the 128 output voxels shifted by the tap,
//    zero-filled outside the volume (the tensor map's pixel box corners are
//    -1 on every axis, i.e. a padding of one cell; the load's coordinates are
//    the first voxel's position minus one, the offsets are the tap);
//  * B: one tiled TMA load per part brings the tap's weights w[co][tap][ci];
//  * both arrive swizzled (32, 64 or 128 B, the part's row width) in the
//    K-major layout the MMA descriptors describe; channel counts that are not
//    a power of two are split into parts of 64, 32 and 16 channels;
//  * one thread issues the loads TMA_STAGES taps ahead and the tap's cin/16
//    MMAs (K = 16 each, the descriptor start advanced by 32 B inside the
//    swizzle atom), committing each tap to its stage's "empty" mbarrier; the
//    stage is reloaded once its MMAs completed.
// The epilogue (TMEM -> registers -> bias/activation/mask -> BF16) is the one
// of nn_tc.cu.  Every mbarrier wait is bounded (about a second); on a timeout
// the CTA records an error flag (nn_tma_take_error), waits (bounded) for the
// copies and MMAs it issued, frees its tensor memory and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

#include "../../include/lbm_nn.h"
#include "lbm_internal.h"
#include "nn_act.cuh"

namespace {
typedef __nv_bfloat16 bf16;

constexpr int TMA_M = 128;
constexpr int TMA_THREADS = 128;
constexpr int TMA_STAGES = 4;
constexpr int TMA_MAX_PARTS = 2;
constexpr long long TMA_WAIT_CYCLES = 2000000000LL;   // about 1 s at 2 GHz

__device__ int g_tma_error;

struct TmaConvArgs {
    CUtensorMap a[TMA_MAX_PARTS];   // im2col maps of the input, one per channel part
    CUtensorMap b[TMA_MAX_PARTS];   // tiled maps of the weights [cout][27][cin], one per part
    int nparts;
    int pw[TMA_MAX_PARTS];          // part widths (16, 32 or 64 channels)
    int poff[TMA_MAX_PARTS];        // first channel of each part
    uint32_t aoff[TMA_MAX_PARTS];   // byte offsets of the parts inside a stage (1024-aligned)
    uint32_t boff[TMA_MAX_PARTS];
    uint32_t stage_bytes;           // a multiple of 1024
    uint32_t stage_tx;              // bytes the TMA writes per stage
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool tma_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > TMA_WAIT_CYCLES) return false;
    }
}

// UMMA layout code of a K-major swizzled operand whose rows are `span` bytes.
__host__ __device__ constexpr uint32_t layout_code(int span) { return span == 128 ? 2u : (span == 64 ? 4u : 6u); }

// Shared-memory matrix descriptor of a K-major swizzled operand: rows of
// `span` bytes, 8-row groups `8 span` bytes apart (SBO); LBO is not used by
// swizzled K-major layouts (encoded as 1).
__device__ __forceinline__ uint64_t sw_desc(uint32_t addr, int span) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(((8u * (uint32_t)span) >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)layout_code(span) << 61;
    return d;
}

__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
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

// Issue the loads of tap t into the stage at `sbase` (one thread).
__device__ __forceinline__ void issue_tap(const TmaConvArgs& P, int t, uint32_t sbase, uint64_t* full, int w0, int h0,
                                          int d0, int n0) {
    const int tz = t / 9, ty = (t / 3) % 3, tx = t % 3;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(full)), "r"(P.stage_tx)
                 : "memory");
    const unsigned short ox = (unsigned short)tx, oy = (unsigned short)ty, oz = (unsigned short)tz;
    for (int p = 0; p < P.nparts; ++p) {
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.im2col.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4, %5, %6}], [%7], {%8, %9, %10};" ::"r"(sbase + P.aoff[p]),
            "l"(&P.a[p]), "r"(P.poff[p]), "r"(w0 - 1), "r"(h0 - 1), "r"(d0 - 1), "r"(n0), "r"(su32(full)), "h"(ox),
            "h"(oy), "h"(oz)
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(sbase + P.boff[p]),
            "l"(&P.b[p]), "r"(P.poff[p]), "r"(t), "r"(0), "r"(su32(full))
            : "memory");
    }
}

// MODE as conv3d_tc_kernel: 0 relu(conv + bias); 1 conv * (mask > 0); 2 pre =
// conv + bias, out = gelu(pre); 3 conv * gelu'(mask).
template <int COUT, int MODE>
__global__ void __launch_bounds__(TMA_THREADS) conv3d_tma_kernel(const __grid_constant__ TmaConvArgs P,
                                                                const float* __restrict__ bias,
                                                                const bf16* __restrict__ mask, bf16* __restrict__ out,
                                                                bf16* __restrict__ pre, int N, int D, int H, int W) {
    constexpr uint32_t NCOL = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);
    constexpr uint32_t IDESC = idesc_f16(TMA_M, COUT);
    extern __shared__ unsigned char dsmem[];
    __shared__ __align__(8) uint64_t s_full[TMA_STAGES];
    __shared__ __align__(8) uint64_t s_empty[TMA_STAGES];
    __shared__ __align__(8) uint64_t s_done;
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (su32(dsmem) + 1023u) & ~1023u;   // swizzle atoms want 1024-byte alignment
    if (tid == 0) {
        for (int s = 0; s < TMA_STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_full[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_empty[s])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_done)) : "memory");
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_taddr)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;

    const int64_t nvox = (int64_t)N * D * H * W;
    const int64_t v0 = (int64_t)blockIdx.x * TMA_M;
    if (tid == 0) {
        int w0 = (int)(v0 % W);
        int64_t q = v0 / W;
        const int h0 = (int)(q % H);
        q /= H;
        const int d0 = (int)(q % D);
        const int n0 = (int)(q / D);
        int issued = 0, consumed = 0;
        bool fail = false;
        for (; issued < TMA_STAGES && issued < 27; ++issued)
            issue_tap(P, issued, base + (uint32_t)issued * P.stage_bytes, &s_full[issued], w0, h0, d0, n0);
        for (int t = 0; t < 27 && !fail; ++t) {
            const int s = t % TMA_STAGES;
            const uint32_t par = (uint32_t)((t / TMA_STAGES) & 1);
            if (!tma_wait(&s_full[s], par)) { fail = true; break; }
            ++consumed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sb = base + (uint32_t)s * P.stage_bytes;
            for (int p = 0; p < P.nparts; ++p) {
                const int span = P.pw[p] * 2;
                for (int k = 0; k < P.pw[p] / 16; ++k)
                    mma_f16(taddr, sw_desc(sb + P.aoff[p] + 32u * k, span), sw_desc(sb + P.boff[p] + 32u * k, span),
                            IDESC, (t | p | k) != 0 ? 1u : 0u);
            }
            mma_commit(&s_empty[s]);
            if (t + TMA_STAGES < 27) {
                // the stage is free once this tap's MMAs have read it
                if (!tma_wait(&s_empty[s], par)) { fail = true; break; }
                issue_tap(P, t + TMA_STAGES, sb, &s_full[s], w0, h0, d0, n0);
                ++issued;
            }
        }
        if (fail) {
            // let the copies already issued land before the CTA leaves
            for (int t = consumed; t < issued; ++t) tma_wait(&s_full[t % TMA_STAGES], (uint32_t)((t / TMA_STAGES) & 1));
            s_fail = 1;
        }
        mma_commit(&s_done);   // arrives when every MMA issued above has completed
    }
    __syncthreads();
    const bool done = tma_wait(&s_done, 0);
    if (!done) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int64_t v = v0 + tid;
    const bool live = v < nvox;
    if (!s_fail) {
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);   // this warp's 32 TMEM lanes
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tw + (uint32_t)c0, acc);
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
        atomicExch(&g_tma_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(NCOL) : "memory");
}

// ---------------------------------------------------------------------------
// Weight gradient dW[co][tap][ci] = sum_v g[v][co] in[v + tap][ci] (and the
// bias gradient sum_v g[v][co]) as a GEMM over K = voxels.
//
// Both operands are channels-last in memory, i.e. MN-major for this GEMM, and
// are used in place: D[(tap, ci)][co] with M = 128 rows holding 128 / pw taps
// of one channel part (8 taps of 16 channels, 4 of 32, 2 of 64; the tap slots
// sit one leading-byte offset apart), N = output channels.  A K stage is one
// block of 8 x 4 x 4 voxels: one tiled TMA box of g at the block and, per tap,
// one box of the input at the block shifted by the tap (zero outside the
// volume).  Because g and the inputs share the block's voxel order, the sum
// over K is the sum over voxels.  The last tap group of the first channel part
// always has a free slot (27 is not a multiple of 2, 4 or 8); it holds ones,
// and its rows accumulate sum_v g[v][co], the bias-gradient partial.
// A CTA handles one (channel part, tap group) and WGB_CHUNK blocks; partials
// part[chunk][tap][co][ci] and dbpart[chunk][co] are summed over chunks in a
// fixed order by the reduction kernels of nn_unet.cu.
constexpr int WGB_W = 8, WGB_H = 4, WGB_D = 4;   // one K stage: 128 voxels
constexpr int WGB_CHUNK = 32;                     // blocks (4096 voxels) per CTA
constexpr int WGB_MAX_STAGES = 4;

struct TmaWgradArgs {
    CUtensorMap a[TMA_MAX_PARTS];   // input, tiled 5-D, box (pw, 8, 4, 4, 1), one per channel part
    CUtensorMap g[TMA_MAX_PARTS];   // g, tiled 5-D, box (gw, 8, 4, 4, 1), one per output-channel part
    int nparts, pw[TMA_MAX_PARTS], poff[TMA_MAX_PARTS];
    int ngparts, gw[TMA_MAX_PARTS], goff[TMA_MAX_PARTS];
    int kinds0;                     // tap groups of channel part 0; the other kinds belong to part 1
    uint32_t boff[TMA_MAX_PARTS];   // byte offsets of the g parts in a stage (after the 32 KB of A)
    uint32_t stage_bytes;           // a multiple of 1024
    int stages;                     // ring depth, 2..WGB_MAX_STAGES
    int nbw, nbh, nbd;              // blocks along W, H, D
    int64_t nblocks;
    int cin, cout;
};

__host__ __device__ constexpr uint32_t idesc_mn(int m, int n) { return idesc_f16(m, n) | (1u << 15) | (1u << 16); }

__device__ __forceinline__ uint64_t mn_desc(uint32_t addr, uint32_t lbo, uint32_t sbo, int span) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)layout_code(span) << 61;
    return d;
}

// Byte offset of 16-byte chunk c of row r in a swizzled K-row-major tile whose rows are `span`
// bytes (1024-aligned base): the chunk index is XORed with the row bits of the swizzle pattern.
__device__ __forceinline__ uint32_t swz(uint32_t r, uint32_t c, uint32_t span) {
    return r * span + ((c ^ ((r * span >> 7) & (span / 16u - 1u))) << 4);
}

template <int COUT>
__global__ void __launch_bounds__(TMA_THREADS) conv3d_wgrad_tma_kernel(const __grid_constant__ TmaWgradArgs P,
                                                                      float* __restrict__ part,
                                                                      float* __restrict__ dbpart) {
    constexpr uint32_t NCOL = COUT <= 32 ? 32 : 64;
    extern __shared__ unsigned char dsmem[];
    __shared__ __align__(8) uint64_t s_full[WGB_MAX_STAGES];
    __shared__ __align__(8) uint64_t s_empty[WGB_MAX_STAGES];
    __shared__ __align__(8) uint64_t s_done;
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (su32(dsmem) + 1023u) & ~1023u;
    unsigned char* gbase = dsmem + (base - su32(dsmem));
    const int kind = blockIdx.x;
    const int64_t chunk = blockIdx.y;
    const int prt = kind < P.kinds0 ? 0 : 1;
    const int grp = prt ? kind - P.kinds0 : kind;
    const int pw = P.pw[prt];
    const uint32_t span = 2u * (uint32_t)pw;
    const int tg = 128 / pw;                       // tap slots in M
    const int tap0 = grp * tg;
    const int ntap = min(tg, 27 - tap0);
    const int ones = (prt == 0 && tap0 + tg >= 27) ? ntap : -1;
    const int64_t b0 = chunk * WGB_CHUNK;
    const int nst = (int)min((int64_t)WGB_CHUNK, P.nblocks - b0);
    const int stages = P.stages;

    // free tap slots: zeros, or ones in the bias slot (never written by the TMA)
    for (int st = 0; st < stages; ++st)
        for (int sl = ntap; sl < tg; ++sl) {
            uint4* dst = reinterpret_cast<uint4*>(gbase + (size_t)st * P.stage_bytes + (size_t)sl * 128 * span);
            const uint32_t v = sl == ones ? 0x3F803F80u : 0u;   // two BF16 ones
            for (uint32_t e = tid; e < 128u * span / 16u; e += TMA_THREADS) dst[e] = make_uint4(v, v, v, v);
        }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) {
        for (int st = 0; st < WGB_MAX_STAGES; ++st) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_full[st])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_empty[st])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_done)) : "memory");
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_taddr)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;

    if (tid == 0) {
        uint32_t tx = (uint32_t)ntap * 128u * span;
        for (int q = 0; q < P.ngparts; ++q) tx += 128u * 2u * (uint32_t)P.gw[q];
        auto issue = [&](int st, int sl) {
            int64_t b = b0 + st;
            const int bw = (int)(b % P.nbw);
            b /= P.nbw;
            const int bh = (int)(b % P.nbh);
            b /= P.nbh;
            const int bd = (int)(b % P.nbd);
            const int n = (int)(b / P.nbd);
            const int w0 = bw * WGB_W, h0 = bh * WGB_H, d0 = bd * WGB_D;
            const uint32_t sb = base + (uint32_t)sl * P.stage_bytes;
            const uint32_t bar = su32(&s_full[sl]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx) : "memory");
            for (int j = 0; j < ntap; ++j) {
                const int t = tap0 + j, tz = t / 9, ty = (t / 3) % 3, txo = t % 3;
                asm volatile(
                    "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(sb + (uint32_t)j * 128u * span),
                    "l"(&P.a[prt]), "r"(P.poff[prt]), "r"(w0 + txo - 1), "r"(h0 + ty - 1), "r"(d0 + tz - 1), "r"(n),
                    "r"(bar)
                    : "memory");
            }
            for (int q = 0; q < P.ngparts; ++q)
                asm volatile(
                    "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(sb + P.boff[q]),
                    "l"(&P.g[q]), "r"(P.goff[q]), "r"(w0), "r"(h0), "r"(d0), "r"(n), "r"(bar)
                    : "memory");
        };
        int issued = 0, consumed = 0;
        bool fail = false;
        const int lag = stages >= 3 ? 1 : 0;
        for (; issued < stages && issued < nst; ++issued) issue(issued, issued);
        for (int st = 0; st < nst; ++st) {
            const int sl = st % stages;
            if (!tma_wait(&s_full[sl], (uint32_t)((st / stages) & 1))) { fail = true; break; }
            ++consumed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = base + (uint32_t)sl * P.stage_bytes;
#pragma unroll 1
            for (int kk = 0; kk < 8; ++kk) {   // K = 16 voxels per MMA: two 8-row groups
                const uint64_t ad = mn_desc(sa + (uint32_t)kk * 16u * span, 128u * span, 8u * span, (int)span);
                for (int q = 0; q < P.ngparts; ++q) {
                    const uint32_t gs = 2u * (uint32_t)P.gw[q];
                    const uint64_t bd = mn_desc(sa + P.boff[q] + (uint32_t)kk * 16u * gs, 8u * gs, 8u * gs, (int)gs);
                    mma_f16(taddr + (uint32_t)P.goff[q], ad, bd, idesc_mn(128, P.gw[q]), (st | kk) != 0 ? 1u : 0u);
                }
            }
            mma_commit(&s_empty[sl]);
            // refill the slot of stage r = st - lag once its MMAs completed; with three or more
            // slots the previous stage's (lag 1), so that two stages of MMAs stay queued
            const int r = st - lag;
            if (r >= 0 && r + stages < nst) {
                const int ps = r % stages;
                if (!tma_wait(&s_empty[ps], (uint32_t)((r / stages) & 1))) { fail = true; break; }
                issue(r + stages, ps);
                ++issued;
            }
        }
        if (fail) {
            for (int st = consumed; st < issued; ++st)
                tma_wait(&s_full[st % stages], (uint32_t)((st / stages) & 1));
            s_fail = 1;
        }
        mma_commit(&s_done);
    }
    __syncthreads();
    if (!tma_wait(&s_done, 0)) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const int slot = tid / pw, cil = tid % pw;
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tw + (uint32_t)c0, acc);
            if (slot < ntap) {
                float* dst = part + ((chunk * 27 + tap0 + slot) * P.cout + c0) * P.cin + P.poff[prt] + cil;
#pragma unroll
                for (int q = 0; q < 16; ++q) dst[(int64_t)q * P.cin] = acc[q];
            } else if (slot == ones && cil == 0) {
#pragma unroll
                for (int q = 0; q < 16; ++q) dbpart[chunk * P.cout + c0 + q] = acc[q];
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_tma_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(NCOL) : "memory");
}

// ---------------------------------------------------------------------------
// Narrow layers (cin x cout small enough for all 27 taps of weights to stay in
// shared memory): one CTA computes TD tiles of 8 (w) x 16 (h) voxels at depths
// d0 .. d0+TD-1 (M = 128 per tile, one TMEM accumulator each) from a single
// halo block of 10 x 18 x (TD + 2) input voxels.  The halo and the weights are
// fetched with coalesced 16-byte cp.async (zero-filled outside the volume)
// into the no-swizzle K-major layout of the MMA: 8-channel planes
// [c8][z][y][x][8], so the A operand of every tap is the same buffer seen
// through a descriptor whose start moves by the tap's offset (rows: 8
// consecutive x = one 128-byte core matrix; row groups: y, 160 bytes apart;
// K chunks: planes).  Weights sit as [tap][c8][co][8].
constexpr int HB_W = 8, HB_H = 16;               // tile of one M = 128 accumulator
constexpr int HB_XW = HB_W + 2, HB_YH = HB_H + 2;

struct HaloArgs {
    int N, D, H, W, cin, td;
    int ntw, nth, ntd;                             // tiles along W, H, D (td deep)
    uint32_t plane;                                // bytes of one 8-channel halo plane
    uint32_t wbase;                                // byte offset of the weights in shared memory
    uint32_t ncol;                                 // allocated TMEM columns (power of two)
};

__device__ __forceinline__ uint64_t plain_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

template <int COUT, int MODE>
__global__ void __launch_bounds__(TMA_THREADS) conv3d_halo_kernel(const HaloArgs P, const bf16* __restrict__ in,
                                                                 const bf16* __restrict__ w,
                                                                 const float* __restrict__ bias,
                                                                 const bf16* __restrict__ mask,
                                                                 bf16* __restrict__ out, bf16* __restrict__ pre) {
    constexpr uint32_t NPER = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);   // columns per accumulator
    constexpr uint32_t IDESC = idesc_f16(TMA_M, COUT);
    extern __shared__ unsigned char dsmem[];
    __shared__ __align__(8) uint64_t s_done;
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (su32(dsmem) + 127u) & ~127u;
    const int kc8 = P.cin >> 3;
    int64_t t = blockIdx.x;
    const int tw = (int)(t % P.ntw);
    t /= P.ntw;
    const int th = (int)(t % P.nth);
    t /= P.nth;
    const int tdd = (int)(t % P.ntd);
    const int n = (int)(t / P.ntd);
    const int w0 = tw * HB_W, h0 = th * HB_H, d0 = tdd * P.td;
    const int zd = P.td + 2;

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_done)) : "memory");
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_taddr)),
                     "r"(P.ncol)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // halo: piece e = ((z * 18 + y) * 10 + x) * kc8 + c8 (consecutive threads: consecutive 16 bytes in memory)
    const int npieces = zd * HB_YH * HB_XW * kc8;
    for (int e = tid; e < npieces; e += TMA_THREADS) {
        const int c8 = e % kc8;
        int r = e / kc8;
        const int x = r % HB_XW;
        r /= HB_XW;
        const int y = r % HB_YH;
        const int z = r / HB_YH;
        const int gx = w0 - 1 + x, gy = h0 - 1 + y, gz = d0 - 1 + z;
        const bool ok = (unsigned)gx < (unsigned)P.W && (unsigned)gy < (unsigned)P.H && (unsigned)gz < (unsigned)P.D;
        const bf16* src = ok ? in + ((((int64_t)n * P.D + gz) * P.H + gy) * P.W + gx) * P.cin + c8 * 8 : in;
        cp16(base + (uint32_t)c8 * P.plane + (uint32_t)((z * HB_YH + y) * HB_XW + x) * 16u, src, ok);
    }
    // weights: piece e = (co * 27 + tap) * kc8 + c8 (the order of w in memory)
    const int wpieces = COUT * 27 * kc8;
    for (int e = tid; e < wpieces; e += TMA_THREADS) {
        const int c8 = e % kc8;
        const int r = e / kc8;
        const int tap = r % 27, co = r / 27;
        cp16(base + P.wbase + ((uint32_t)(tap * kc8 + c8) * COUT + co) * 16u, w + (int64_t)e * 8, true);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;

    if (tid == 0) {
        for (int dz = 0; dz < P.td; ++dz)
            for (int tap = 0; tap < 27; ++tap) {
                const int tz = tap / 9, ty = (tap / 3) % 3, tx = tap % 3;
                const uint32_t a0 = base + (uint32_t)(((dz + tz) * HB_YH + ty) * HB_XW + tx) * 16u;
                const uint32_t b0 = base + P.wbase + (uint32_t)(tap * kc8) * COUT * 16u;
                for (int kk = 0; kk < kc8 / 2; ++kk)
                    mma_f16(taddr + (uint32_t)dz * NPER,
                            plain_desc(a0 + (uint32_t)(2 * kk) * P.plane, P.plane, HB_XW * 16u),
                            plain_desc(b0 + (uint32_t)(2 * kk) * COUT * 16u, COUT * 16u, 128u), IDESC,
                            (tap | kk) != 0 ? 1u : 0u);
            }
        mma_commit(&s_done);
    }
    __syncthreads();
    if (!tma_wait(&s_done, 0)) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const int hx = tid & 7, hy = tid >> 3;           // row m = tid: (h, w) = (m / 8, m % 8)
        const int gx = w0 + hx, gy = h0 + hy;
        const uint32_t twarp = taddr + ((uint32_t)(warp * 32) << 16);
        for (int dz = 0; dz < P.td; ++dz) {
            const int gz = d0 + dz;
            const bool live = gx < P.W && gy < P.H && gz < P.D;
            const int64_t v = (((int64_t)n * P.D + gz) * P.H + gy) * P.W + gx;
#pragma unroll
            for (int c0 = 0; c0 < COUT; c0 += 16) {
                float acc[16];
                tmem_ld16(twarp + (uint32_t)dz * NPER + (uint32_t)c0, acc);
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
        }
    } else if (tid == 0) {
        atomicExch(&g_tma_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(P.ncol) : "memory");
}

// ---------------------------------------------------------------------------
// Warp-specialised weight gradient for layers whose input and output are one
// channel part each (16, 32 or 64 channels): the same GEMM, tap groups, ones
// slot and partials as conv3d_wgrad_tma_kernel, but each 8 x 4 x 4 block is
// loaded once -- one dense TMA box of the 10 x 6 x 6 input halo and one of g
// (no swizzle) -- and a CTA runs all tap groups of its blocks, one TMEM
// accumulator per group.
//   warp 4, lane 0: TMA producer (two boxes per block, two buffers) and MMA
//     issuer (8 K = 16 steps per block and group, two operand buffers);
//   warps 0-3: build the operand buffer of each (block, group) step from the
//     halo -- tap slot j row r is the halo voxel r shifted by the tap, written
//     in the swizzled MN-major layout -- plus the g operand, then the epilogue.
// mbarriers between the roles: tfull (TMA -> copy), tempty (copy -> producer,
// 128 arrivals), ofull (copy -> MMA, 128 arrivals), oempty (MMA commit ->
// copy), done.  Every wait is bounded; a timeout records the error flag and
// the roles leave their loops, the producer first waiting (bounded) for the
// loads it issued.
constexpr int WS_THREADS = 160;

struct WsArgs {
    CUtensorMap halo;               // input, tiled 5-D (cin, W, H, D, N), box (cin, 10, 6, 6, 1), no swizzle
    CUtensorMap gmap;               // g, tiled 5-D (cout, W, H, D, N), box (cout, 8, 4, 4, 1), no swizzle
    int cin, cout, tg, ngroups;     // tap slots per group (128 / cin), groups (ceil(27 / tg))
    uint32_t hbytes;                // bytes of the halo box
    uint32_t tbytes;                // bytes of one TMA buffer (halo then g), 1024-aligned
    uint32_t obytes;                // bytes of one operand buffer (32 KB of tap slots + g), 1024-aligned
    uint32_t ncol;                  // TMEM columns (power of two >= ngroups x cout)
    int shift[27];                  // byte offset of tap t's shift inside the halo
    int nbw, nbh, nbd;
    int64_t nblocks;
    int chunk_blocks;               // blocks per CTA (and per partial)
};

template <int COUT>
__global__ void __launch_bounds__(WS_THREADS, 1) conv3d_wgrad_ws_kernel(const __grid_constant__ WsArgs P,
                                                                    float* __restrict__ part,
                                                                    float* __restrict__ dbpart) {
    extern __shared__ unsigned char dsmem[];
    __shared__ __align__(8) uint64_t s_tfull[2], s_tempty[2], s_ofull[2], s_oempty[2], s_done;
    __shared__ uint32_t s_taddr;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (su32(dsmem) + 1023u) & ~1023u;
    const uint32_t obase = base + 2u * P.tbytes;
    const int64_t chunk = blockIdx.x;
    const int64_t b0 = chunk * P.chunk_blocks;
    const int nb = (int)min((int64_t)P.chunk_blocks, P.nblocks - b0);
    const int pw = P.cin, tg = P.tg, ng = P.ngroups;
    const uint32_t span = 2u * (uint32_t)pw;
    const uint32_t gs = 2u * (uint32_t)COUT;
    const int ntap_last = 27 - (ng - 1) * tg;            // taps of the last group; its slot ntap_last holds ones

    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_tfull[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(su32(&s_tempty[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(su32(&s_ofull[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_oempty[b])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&s_done)) : "memory");
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_taddr)),
                     "r"(P.ncol)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_taddr;
    const int nsteps = nb * ng;

    if (warp == 4) {
        if ((tid & 31) == 0) {   // producer + MMA issuer
            const uint32_t tx = P.hbytes + 128u * gs;
            auto issue = [&](int b) {
                int64_t q = b0 + b;
                const int bw = (int)(q % P.nbw);
                q /= P.nbw;
                const int bh = (int)(q % P.nbh);
                q /= P.nbh;
                const int bd = (int)(q % P.nbd);
                const int n = (int)(q / P.nbd);
                const int w0 = bw * WGB_W, h0 = bh * WGB_H, d0 = bd * WGB_D;
                const uint32_t tb = base + (uint32_t)(b & 1) * P.tbytes;
                const uint32_t bar = su32(&s_tfull[b & 1]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx) : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(tb),
                    "l"(&P.halo), "r"(0), "r"(w0 - 1), "r"(h0 - 1), "r"(d0 - 1), "r"(n), "r"(bar)
                    : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(tb + P.hbytes),
                    "l"(&P.gmap), "r"(0), "r"(w0), "r"(h0), "r"(d0), "r"(n), "r"(bar)
                    : "memory");
            };
            int issued = 0, landed = 0;
            bool fail = false;
            for (; issued < 2 && issued < nb; ++issued) issue(issued);
            for (int st = 0; st < nsteps && !fail; ++st) {
                const int b = st / ng, gi = st - b * ng, ob = st & 1;
                if (!tma_wait(&s_ofull[ob], (uint32_t)((st >> 1) & 1))) { fail = true; break; }
                if (gi == 0) landed = b + 1;   // the copy warps saw block b's loads complete
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = obase + (uint32_t)ob * P.obytes;
                const uint32_t acc = taddr + (uint32_t)(gi * COUT);
#pragma unroll 1
                for (int kk = 0; kk < 8; ++kk) {
                    const uint64_t ad = mn_desc(sa + (uint32_t)kk * 16u * span, 128u * span, 8u * span, (int)span);
                    const uint64_t bdsc =
                        mn_desc(sa + 32768u + (uint32_t)kk * 16u * gs, 8u * gs, 8u * gs, (int)gs);
                    mma_f16(acc, ad, bdsc, idesc_mn(128, COUT), (b | kk) != 0 ? 1u : 0u);
                }
                mma_commit(&s_oempty[ob]);
                if (gi == ng - 1 && b + 2 < nb) {   // block b's halo is no longer read: load block b + 2 there
                    if (!tma_wait(&s_tempty[b & 1], (uint32_t)((b >> 1) & 1))) { fail = true; break; }
                    issue(b + 2);
                    ++issued;
                }
            }
            if (fail) {
                for (int b = landed; b < issued; ++b) tma_wait(&s_tfull[b & 1], (uint32_t)((b >> 1) & 1));
                s_fail = 1;
                atomicExch(&g_tma_error, 1);
            }
            mma_commit(&s_done);
        }
    } else {
        // copy warps: the per-thread chunks of a step are fixed; tap t adds P.shift[t] to the source
        const int csh = pw == 64 ? 3 : (pw == 32 ? 2 : 1);
        // packed: source offset in the halo (< 46 KB) | destination offset in the tap slots (< 32 KB) << 16
        uint32_t pk[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int e = tid + k * 128;
            const int c = e & ((1 << csh) - 1);
            const int r = (e >> csh) & 127;
            const int j = e >> (7 + csh);                     // tap slot (< tg)
            const int x = r & 7, y = (r >> 3) & 3, z = r >> 5;   // voxel of the block; halo origin at -1
            const uint32_t src = (uint32_t)((z * 6 + y) * 10 + x) * span + (uint32_t)c * 16u;
            const uint32_t dst = (uint32_t)j * 128u * span + swz((uint32_t)r, (uint32_t)c, span);
            pk[k] = src | (dst << 16);
        }
        const int gch = COUT / 8;                             // g chunks per row
        bool fail = false;
        for (int st = 0; st < nsteps; ++st) {
            const int b = st / ng, gi = st - b * ng, ob = st & 1;
            if (gi == 0 && !tma_wait(&s_tfull[b & 1], (uint32_t)((b >> 1) & 1))) { fail = true; break; }
            if (st >= 2 && !tma_wait(&s_oempty[ob], (uint32_t)(((st - 2) >> 1) & 1))) { fail = true; break; }
            const uint32_t tsh = base + (uint32_t)(b & 1) * P.tbytes;
            const uint32_t osh = obase + (uint32_t)ob * P.obytes;
            const int ntap = gi == ng - 1 ? ntap_last : tg;
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const int j = (tid + k * 128) >> (7 + csh);
                if (j < ntap) {
                    uint32_t v0, v1, v2, v3;
                    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                                 : "=r"(v0), "=r"(v1), "=r"(v2), "=r"(v3)
                                 : "r"(tsh + (pk[k] & 0xFFFFu) + (uint32_t)P.shift[gi * tg + j]));
                    asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(osh + (pk[k] >> 16)), "r"(v0), "r"(v1),
                                 "r"(v2), "r"(v3)
                                 : "memory");
                } else if (gi == ng - 1 && j == ntap) {          // the ones slot of the last group
                    const uint32_t one = 0x3F803F80u;
                    asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(osh + (pk[k] >> 16)), "r"(one) : "memory");
                }
            }
            for (int e = tid; e < 128 * gch; e += 128) {        // g operand: row r, chunk c8
                const int c8 = e % gch, r = e / gch;
                uint32_t v0, v1, v2, v3;
                asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                             : "=r"(v0), "=r"(v1), "=r"(v2), "=r"(v3)
                             : "r"(tsh + P.hbytes + (uint32_t)r * gs + (uint32_t)c8 * 16u));
                asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(osh + 32768u + swz((uint32_t)r, (uint32_t)c8, gs)),
                             "r"(v0), "r"(v1), "r"(v2), "r"(v3)
                             : "memory");
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&s_ofull[ob])) : "memory");
            if (gi == ng - 1)   // done reading block b's halo and g
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&s_tempty[b & 1])) : "memory");
        }
        if (fail) {
            s_fail = 1;
            if (tid == 0) atomicExch(&g_tma_error, 1);
        }
        if (!tma_wait(&s_done, 0)) s_fail = 1;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (s_fail) {
        if (tid == 0) atomicExch(&g_tma_error, 1);
    } else if (warp < 4) {
        const int sl = tid / pw, cil = tid % pw;
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);
        for (int gi = 0; gi < ng; ++gi) {
            const int ntap = gi == ng - 1 ? ntap_last : tg;
#pragma unroll
            for (int c0 = 0; c0 < COUT; c0 += 16) {
                float acc[16];
                tmem_ld16(tw + (uint32_t)(gi * COUT + c0), acc);
                if (sl < ntap) {
                    float* dst = part + ((chunk * 27 + gi * tg + sl) * COUT + c0) * P.cin + cil;
#pragma unroll
                    for (int q = 0; q < 16; ++q) dst[(int64_t)q * P.cin] = acc[q];
                } else if (gi == ng - 1 && sl == ntap && cil == 0) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) dbpart[chunk * COUT + c0 + q] = acc[q];
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(P.ncol) : "memory");
}

// Driver entry points for the tensor maps, resolved through the runtime.
typedef CUresult(CUDAAPI* EncIm2col)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                     const cuuint64_t*, const int*, const int*, cuuint32_t, cuuint32_t,
                                     const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                     CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
typedef CUresult(CUDAAPI* EncTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncIm2col g_enc_im2col = nullptr;
EncTiled g_enc_tiled = nullptr;
std::once_flag g_enc_once;

bool encoders() {
    std::call_once(g_enc_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeIm2col", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_enc_im2col = (EncIm2col)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_enc_tiled = (EncTiled)f;
    });
    return g_enc_im2col && g_enc_tiled;
}

CUtensorMapSwizzle swizzle_of(int span) {
    return span == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : (span == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

template <int COUT, int MODE>
int launch_tma(const TmaConvArgs& P, const float* bias, const bf16* mask, bf16* out, bf16* pre, int n, int d, int h,
               int wd, cudaStream_t s) {
    const size_t smem = (size_t)TMA_STAGES * P.stage_bytes + 1024;
    auto k = conv3d_tma_kernel<COUT, MODE>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA,
                           "lbm_nn_conv3d (TMA): shared memory attribute refused for " + std::to_string(smem) + " bytes");
    const int64_t nvox = (int64_t)n * d * h * wd;
    const int grid = (int)((nvox + TMA_M - 1) / TMA_M);
    k<<<grid, TMA_THREADS, smem, s>>>(P, bias, mask, out, pre, n, d, h, wd);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_tma_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace

// The TMA path handles cin in {16, 32, 48, 64, 80, 96, 128} (one or two parts)
// and cout in {16, 32, 48, 64, 96}; LBM_NN_TMA=0 in the environment selects the
// thread-staged kernel of nn_tc.cu instead.
bool nn_tma_usable(int cin, int cout) {
    static const bool on = [] {
        const char* e = getenv("LBM_NN_TMA");
        return !(e && e[0] == '0');
    }();
    const bool cin_ok = cin == 16 || cin == 32 || cin == 48 || cin == 64 || cin == 80 || cin == 96 || cin == 128;
    const bool cout_ok = cout == 16 || cout == 32 || cout == 48 || cout == 64 || cout == 96;
    return on && cin_ok && cout_ok && encoders();
}

int nn_conv3d_tma(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre, int n, int d,
                  int h, int wd, int cin, int cout, int mode, cudaStream_t s) {
    if (!encoders()) return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d (TMA): tensor-map entry points unavailable");
    TmaConvArgs P{};
    // channel parts: 64, 32 and 16 wide, at most two
    int rest = cin, off = 0;
    P.nparts = 0;
    while (rest > 0) {
        const int pw = rest >= 64 ? 64 : (rest >= 32 ? 32 : 16);
        if (P.nparts == TMA_MAX_PARTS) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d (TMA): unsupported cin");
        P.pw[P.nparts] = pw;
        P.poff[P.nparts] = off;
        ++P.nparts;
        off += pw;
        rest -= pw;
    }
    uint32_t at = 0;
    P.stage_tx = 0;
    for (int p = 0; p < P.nparts; ++p) {
        const uint32_t span = 2u * (uint32_t)P.pw[p];
        P.aoff[p] = at;
        at += ((uint32_t)TMA_M * span + 1023u) & ~1023u;
        P.boff[p] = at;
        at += ((uint32_t)cout * span + 1023u) & ~1023u;
        P.stage_tx += (uint32_t)TMA_M * span + (uint32_t)cout * span;
    }
    P.stage_bytes = at;
    for (int p = 0; p < P.nparts; ++p) {
        const int span = 2 * P.pw[p];
        const cuuint64_t adim[5] = {(cuuint64_t)cin, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
        const cuuint64_t astr[4] = {(cuuint64_t)cin * 2, (cuuint64_t)wd * cin * 2, (cuuint64_t)h * wd * cin * 2,
                                    (cuuint64_t)d * h * wd * cin * 2};
        const int lo[3] = {-1, -1, -1}, hi[3] = {-1, -1, -1};
        const cuuint32_t es[5] = {1, 1, 1, 1, 1};
        CUresult r = g_enc_im2col(&P.a[p], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), adim, astr, lo,
                                  hi, (cuuint32_t)P.pw[p], TMA_M, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(span),
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d (TMA): im2col tensor map, error " + std::to_string((int)r));
        const cuuint64_t bdim[3] = {(cuuint64_t)cin, 27, (cuuint64_t)cout};
        const cuuint64_t bstr[2] = {(cuuint64_t)cin * 2, (cuuint64_t)27 * cin * 2};
        const cuuint32_t box[3] = {(cuuint32_t)P.pw[p], 1, (cuuint32_t)cout};
        const cuuint32_t bes[3] = {1, 1, 1};
        r = g_enc_tiled(&P.b[p], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(w), bdim, bstr, box, bes,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(span), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d (TMA): weight tensor map, error " + std::to_string((int)r));
    }
    const float* B = bias;
    const bf16* M = (const bf16*)mask;
    bf16* O = (bf16*)out;
    bf16* Pr = (bf16*)pre;
#define LBM_TMA(C)                                                          \
    case C:                                                                 \
        switch (mode) {                                                     \
        case 0: return launch_tma<C, 0>(P, B, M, O, Pr, n, d, h, wd, s);    \
        case 1: return launch_tma<C, 1>(P, B, M, O, Pr, n, d, h, wd, s);    \
        case 2: return launch_tma<C, 2>(P, B, M, O, Pr, n, d, h, wd, s);    \
        default: return launch_tma<C, 3>(P, B, M, O, Pr, n, d, h, wd, s);   \
        }
    switch (cout) {
        LBM_TMA(16) LBM_TMA(32) LBM_TMA(48) LBM_TMA(64) LBM_TMA(96)
    }
#undef LBM_TMA
    return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d (TMA): unsupported cout");
}

// Shared memory of the halo kernel for td tiles deep.
static size_t halo_smem(int cin, int cout, int td) {
    const size_t plane = (size_t)(td + 2) * HB_YH * HB_XW * 16;
    return plane * (cin / 8) + (size_t)27 * (cin / 8) * cout * 16 + 128;
}

static int halo_depth() {
    static const int td = [] {
        const char* e = getenv("LBM_NN_HALO_TD");
        const int v = e ? atoi(e) : 2;
        return v >= 1 && v <= 4 ? v : 2;
    }();
    return td;
}

// Narrow layers take the halo kernel: cout in {16, 32, 48, 64}, cin a multiple of
// 16, and the halo plus all weights within 113 KB of shared memory (two CTAs per
// SM).  LBM_NN_HALO=0
// in the environment turns it off.
bool nn_halo_usable(int cin, int cout) {
    static const bool on = [] {
        const char* e = getenv("LBM_NN_HALO");
        return !(e && e[0] == '0');
    }();
    const bool cout_ok = cout == 16 || cout == 32 || cout == 48 || cout == 64;
    return on && cout_ok && cin % 16 == 0 && cin >= 16 && halo_smem(cin, cout, halo_depth()) <= 113 * 1024;
}

template <int COUT, int MODE>
static int launch_halo(const HaloArgs& P, const bf16* in, const bf16* w, const float* bias, const bf16* mask, bf16* out,
                       bf16* pre, size_t smem, cudaStream_t s) {
    auto k = conv3d_halo_kernel<COUT, MODE>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d (halo): shared memory attribute refused");
    const int64_t grid = (int64_t)P.N * P.ntd * P.nth * P.ntw;
    k<<<(unsigned)grid, TMA_THREADS, smem, s>>>(P, in, w, bias, mask, out, pre);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_halo_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int nn_conv3d_halo(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre, int n, int d,
                   int h, int wd, int cin, int cout, int mode, cudaStream_t s) {
    HaloArgs P{};
    P.N = n; P.D = d; P.H = h; P.W = wd; P.cin = cin;
    P.td = halo_depth();
    P.ntw = (wd + HB_W - 1) / HB_W;
    P.nth = (h + HB_H - 1) / HB_H;
    P.ntd = (d + P.td - 1) / P.td;
    P.plane = (uint32_t)(P.td + 2) * HB_YH * HB_XW * 16u;
    P.wbase = P.plane * (uint32_t)(cin / 8);
    const uint32_t nper = cout <= 32 ? 32u : 64u;
    uint32_t nc = 32;
    while (nc < nper * (uint32_t)P.td) nc <<= 1;
    P.ncol = nc;
    const size_t smem = halo_smem(cin, cout, P.td);
    const bf16* I = (const bf16*)in;
    const bf16* Wt = (const bf16*)w;
    const bf16* M = (const bf16*)mask;
    bf16* O = (bf16*)out;
    bf16* Pr = (bf16*)pre;
#define LBM_HALO(C)                                                               \
    case C:                                                                       \
        switch (mode) {                                                           \
        case 0: return launch_halo<C, 0>(P, I, Wt, bias, M, O, Pr, smem, s);      \
        case 1: return launch_halo<C, 1>(P, I, Wt, bias, M, O, Pr, smem, s);      \
        case 2: return launch_halo<C, 2>(P, I, Wt, bias, M, O, Pr, smem, s);      \
        default: return launch_halo<C, 3>(P, I, Wt, bias, M, O, Pr, smem, s);     \
        }
    switch (cout) {
        LBM_HALO(16) LBM_HALO(32) LBM_HALO(48) LBM_HALO(64)
    }
#undef LBM_HALO
    return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d (halo): unsupported cout");
}

// Blocks of the weight-gradient K loop and the chunks they form.
static int64_t wgrad_tma_blocks(int n, int d, int h, int w) {
    return (int64_t)n * ((d + WGB_D - 1) / WGB_D) * ((h + WGB_H - 1) / WGB_H) * ((w + WGB_W - 1) / WGB_W);
}

int64_t nn_wgrad_tma_chunks(int n, int d, int h, int w) {
    return (wgrad_tma_blocks(n, d, h, w) + WGB_CHUNK - 1) / WGB_CHUNK;
}

// The TMA weight gradient takes cin in {16, 32, 48, 64, 80, 96, 128} and cout in
// {16, 32, 48, 64}; LBM_NN_TMA=0 selects the register-staged kernel of nn_tc.cu.
bool nn_wgrad_tma_usable(int cin, int cout) {
    static const bool on = [] {
        const char* e = getenv("LBM_NN_TMA");
        return !(e && e[0] == '0');
    }();
    const bool cin_ok = cin == 16 || cin == 32 || cin == 48 || cin == 64 || cin == 80 || cin == 96 || cin == 128;
    const bool cout_ok = cout == 16 || cout == 32 || cout == 48 || cout == 64;
    return on && cin_ok && cout_ok && encoders();
}

// Partials for nn_wgrad_tma_chunks(n, d, h, w) chunks into part / dbpart.
int nn_wgrad_tma(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int wd, int cin,
                 int cout, cudaStream_t s) {
    if (!encoders()) return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (TMA): tensor-map entry points unavailable");
    TmaWgradArgs P{};
    auto split = [](int c, int* w, int* off) {
        int k = 0, o = 0;
        while (c > 0 && k < TMA_MAX_PARTS) {
            const int pw = c >= 64 ? 64 : (c >= 32 ? 32 : 16);
            w[k] = pw;
            off[k] = o;
            ++k;
            o += pw;
            c -= pw;
        }
        return c == 0 ? k : -1;
    };
    P.nparts = split(cin, P.pw, P.poff);
    P.ngparts = split(cout, P.gw, P.goff);
    if (P.nparts < 1 || P.ngparts < 1) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (TMA): unsupported channels");
    const int tg0 = 128 / P.pw[0];
    P.kinds0 = (27 + tg0 - 1) / tg0;
    const int kinds = P.kinds0 + (P.nparts > 1 ? (27 + 128 / P.pw[1] - 1) / (128 / P.pw[1]) : 0);
    uint32_t at = 128u * 128u * 2u;
    for (int q = 0; q < P.ngparts; ++q) {
        P.boff[q] = at;
        at += (128u * 2u * (uint32_t)P.gw[q] + 1023u) & ~1023u;
    }
    P.stage_bytes = at;
    P.stages = (int)std::min<uint32_t>(WGB_MAX_STAGES, std::max<uint32_t>(2u, (110u * 1024u) / at));
    P.nbw = (wd + WGB_W - 1) / WGB_W;
    P.nbh = (h + WGB_H - 1) / WGB_H;
    P.nbd = (d + WGB_D - 1) / WGB_D;
    P.nblocks = wgrad_tma_blocks(n, d, h, wd);
    P.cin = cin;
    P.cout = cout;
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    for (int p = 0; p < P.nparts; ++p) {
        const cuuint64_t dim[5] = {(cuuint64_t)cin, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
        const cuuint64_t str[4] = {(cuuint64_t)cin * 2, (cuuint64_t)wd * cin * 2, (cuuint64_t)h * wd * cin * 2,
                                   (cuuint64_t)d * h * wd * cin * 2};
        const cuuint32_t box[5] = {(cuuint32_t)P.pw[p], WGB_W, WGB_H, WGB_D, 1};
        CUresult r = g_enc_tiled(&P.a[p], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), dim, str, box, es,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(2 * P.pw[p]), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (TMA): input tensor map, error " + std::to_string((int)r));
    }
    for (int q = 0; q < P.ngparts; ++q) {
        const cuuint64_t dim[5] = {(cuuint64_t)cout, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
        const cuuint64_t str[4] = {(cuuint64_t)cout * 2, (cuuint64_t)wd * cout * 2, (cuuint64_t)h * wd * cout * 2,
                                   (cuuint64_t)d * h * wd * cout * 2};
        const cuuint32_t box[5] = {(cuuint32_t)P.gw[q], WGB_W, WGB_H, WGB_D, 1};
        CUresult r = g_enc_tiled(&P.g[q], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(g), dim, str, box, es,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(2 * P.gw[q]), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (TMA): g tensor map, error " + std::to_string((int)r));
    }
    const int64_t nchunk = nn_wgrad_tma_chunks(n, d, h, wd);
    if (nchunk > 65535) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (TMA): more than 65535 chunks");
    const size_t smem = (size_t)P.stages * P.stage_bytes + 1024;
    const dim3 grid((unsigned)kinds, (unsigned)nchunk);
#define LBM_WGT(C)                                                                                                 \
    case C: {                                                                                                      \
        auto k = conv3d_wgrad_tma_kernel<C>;                                                                       \
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)        \
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (TMA): shared memory attribute refused"); \
        k<<<grid, TMA_THREADS, smem, s>>>(P, part, dbpart);                                                        \
        break;                                                                                                     \
    }
    switch (cout) {
        LBM_WGT(16) LBM_WGT(32) LBM_WGT(48) LBM_WGT(64)
    default:
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (TMA): unsupported cout");
    }
#undef LBM_WGT
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_wgrad_tma_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

// Warp-specialised weight gradient: one-part layers (cin and cout in {16, 32, 64})
// whose accumulators (groups x cout columns) and buffers fit.  It is taken where
// two CTAs fit an SM (113 KB) or cout = 64 > cin: with one CTA per SM the
// TMA-box kernel was faster on 16 -> 32 and 32 -> 32 (2 x 48^3), while on 32 -> 64
// the per-group reload of the 64-channel g made that kernel the slower one.
// LBM_NN_WS=0 in the environment turns it off.
static bool ws_plan(int cin, int cout, WsArgs* P, size_t* smem) {
    if (!(cin == 16 || cin == 32 || cin == 64) || !(cout == 16 || cout == 32 || cout == 64)) return false;
    P->cin = cin;
    P->cout = cout;
    P->tg = 128 / cin;
    P->ngroups = (27 + P->tg - 1) / P->tg;
    if (P->ngroups * cout > 512) return false;
    P->ncol = 32;
    while (P->ncol < (uint32_t)(P->ngroups * cout)) P->ncol <<= 1;
    P->hbytes = 360u * (uint32_t)cin * 2u;
    P->tbytes = (P->hbytes + 128u * 2u * (uint32_t)cout + 1023u) & ~1023u;
    P->obytes = 32768u + ((128u * 2u * (uint32_t)cout + 1023u) & ~1023u);
    for (int t = 0; t < 27; ++t) P->shift[t] = ((t / 9) * 60 + ((t / 3) % 3) * 10 + t % 3) * cin * 2;
    *smem = 2 * (size_t)P->tbytes + 2 * (size_t)P->obytes + 1024;
    return *smem <= 227 * 1024;
}

// Blocks per CTA: enough CTAs for about eight per SM of a 152-SM GPU, 2 to 32 blocks each.
static int ws_chunk_blocks(int64_t nblocks) {
    const int64_t c = (nblocks + 1215) / 1216;
    return (int)std::min<int64_t>(WGB_CHUNK, std::max<int64_t>(2, c));
}

int64_t nn_wgrad_ws_chunks(int n, int d, int h, int w) {
    const int64_t nb = wgrad_tma_blocks(n, d, h, w);
    const int cb = ws_chunk_blocks(nb);
    return (nb + cb - 1) / cb;
}

bool nn_wgrad_ws_usable(int cin, int cout) {
    static const bool on = [] {
        const char* e = getenv("LBM_NN_WS");
        return !(e && e[0] == '0');
    }();
    WsArgs P{};
    size_t smem = 0;
    if (!on || !encoders() || !ws_plan(cin, cout, &P, &smem)) return false;
    return smem <= 113 * 1024 || (cout == 64 && cin < cout);
}

// Partials for nn_wgrad_ws_chunks(n, d, h, w) chunks of the same 8 x 4 x 4 blocks.
int nn_wgrad_ws(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int wd, int cin, int cout,
                cudaStream_t s) {
    if (!encoders()) return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (ws): tensor-map entry points unavailable");
    WsArgs P{};
    size_t smem = 0;
    if (!ws_plan(cin, cout, &P, &smem)) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (ws): unsupported channels");
    P.nbw = (wd + WGB_W - 1) / WGB_W;
    P.nbh = (h + WGB_H - 1) / WGB_H;
    P.nbd = (d + WGB_D - 1) / WGB_D;
    P.nblocks = wgrad_tma_blocks(n, d, h, wd);
    P.chunk_blocks = ws_chunk_blocks(P.nblocks);
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    {
        const cuuint64_t dim[5] = {(cuuint64_t)cin, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
        const cuuint64_t str[4] = {(cuuint64_t)cin * 2, (cuuint64_t)wd * cin * 2, (cuuint64_t)h * wd * cin * 2,
                                   (cuuint64_t)d * h * wd * cin * 2};
        const cuuint32_t box[5] = {(cuuint32_t)cin, 10, 6, 6, 1};
        const CUresult r = g_enc_tiled(&P.halo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), dim, str, box,
                                       es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                       CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (ws): halo tensor map, error " + std::to_string((int)r));
    }
    {
        const cuuint64_t dim[5] = {(cuuint64_t)cout, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
        const cuuint64_t str[4] = {(cuuint64_t)cout * 2, (cuuint64_t)wd * cout * 2, (cuuint64_t)h * wd * cout * 2,
                                   (cuuint64_t)d * h * wd * cout * 2};
        const cuuint32_t box[5] = {(cuuint32_t)cout, WGB_W, WGB_H, WGB_D, 1};
        const CUresult r = g_enc_tiled(&P.gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(g), dim, str, box,
                                       es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                       CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (ws): g tensor map, error " + std::to_string((int)r));
    }
    const int64_t nchunk = nn_wgrad_ws_chunks(n, d, h, wd);
    if (nchunk > 2147483647LL) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (ws): too many chunks");
#define LBM_WS(C)                                                                                                \
    case C: {                                                                                                    \
        auto k = conv3d_wgrad_ws_kernel<C>;                                                                      \
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)      \
            return lbm_set_err(nullptr, LBM_ECUDA, "lbm_nn_conv3d_wgrad (ws): shared memory attribute refused"); \
        k<<<(unsigned)nchunk, WS_THREADS, smem, s>>>(P, part, dbpart);                                           \
        break;                                                                                                   \
    }
    switch (cout) {
        LBM_WS(16) LBM_WS(32) LBM_WS(64)
    default:
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_nn_conv3d_wgrad (ws): unsupported cout");
    }
#undef LBM_WS
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lbm_set_err(nullptr, LBM_ECUDA, std::string("conv3d_wgrad_ws_kernel: ") + cudaGetErrorString(e));
    return LBM_OK;
}

// 1 when a TMA convolution timed out since the last call (cleared on read).
int nn_tma_take_error(int* flag) {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_error, sizeof(int)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_tma_error, &zero, sizeof(int)) != cudaSuccess)
        return LBM_ECUDA;
    *flag = v;
    return LBM_OK;
}
