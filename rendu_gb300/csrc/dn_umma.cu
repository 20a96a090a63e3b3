// 3x3 convolution (forward and data gradient) on the 5th-generation tensor cores: an
// implicit GEMM whose 128 x N tiles accumulate in tensor memory (TMEM) through
// tcgen05.mma, with both operands brought into shared memory by TMA.
//
//   D[m][n] = sum_k A[m][k] B[n][k],  m = output pixel, n = output channel.
//
// A CTA tile is a block of Wb x Hb = 128 pixels of one image (Wb = min(128, the next power
// of two >= the width)). K runs over the 9 taps and, per tap, over 64-channel chunks of
// the input -- first those of input 0, then those of the skip input 1. The A operand of
// one (tap, chunk) is a single tiled TMA box of 64 channels x Wb x Hb pixels at (chunk,
// x0 + dx, y0 + dy, image): the copy engine's zero fill outside the tensor is exactly the
// convolution's zero padding (and the zero channels of a chunk past the channel count).
// The weights are packed to match: K-major rows [Cout][9 x chunks x 64], zero where a
// chunk runs past the channel count; the B operand of a k-block is one 2-D box.
// Both boxes land in the 128-byte-swizzle K-major layout that tcgen05.mma reads (one
// 128-byte row per pixel / output channel, 8-row groups 1024 bytes apart).
//
// Three kernels share that scheme. k_conv_umma takes any tile shape (small images: Wb < 128).
// k_conv_rows takes row tiles (Wb = 128, Hb = 1) and reads one 130-pixel box per kernel row
// for its three horizontal taps. k_conv_fold, used for row tiles whose output fits N <= 85
// channels and whose weights fit in shared memory, moves the three horizontal taps into the
// MMA's N dimension. On the GB300 each tcgen05.mma and tcgen05.commit costs about the same
// whatever its N for these narrow layers (measured: tripling N changed nothing, removing the
// MMAs removed a third of the time), so fewer and wider instructions are what pays.
//
// Each kernel is persistent and warp-specialised: one thread issues the TMA loads into a
// ring of shared-memory stages (full[s]: the stage's bytes have landed; empty[s]: the MMAs
// that read it have completed), one thread issues the MMAs into up to four TMEM
// accumulators (tfull[a]: a tile is complete; tempty[a]: the epilogue has read it back),
// and four epilogue groups of four warps, one group per accumulator, read finished tiles
// with tcgen05.ld (the warp of lane quarter i owns TMEM lanes 32i..32i+31 = tile rows), add
// the bias, apply the ReLU and store BF16 or FP32 NHWC while later tiles accumulate.
//
// Every mbarrier wait is bounded (about 2 s of %globaltimer); a wait that gives up sets
// the status word and its role stops, and the CTA frees its TMEM before it returns. The
// macros DN_FOLD, DN_C32, DN_MAX_STAGES and DN_EPI_GROUPS select layout choices and are
// kept selectable for measurement; the defaults are the measured best.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <string>

#include "dn_net.hpp"

namespace rgb {
namespace dn {

__device__ unsigned g_umma_status;  // nonzero: a bounded wait gave up (RT_ERR_TIMEOUT)

namespace {

constexpr int TM = 128;       // tile rows (pixels): one TMEM lane each
constexpr int KB = 64;        // K per stage: one 128-byte swizzle row of BF16
#ifndef DN_MAX_STAGES
#define DN_MAX_STAGES 8
#endif
constexpr int MAX_STAGES = DN_MAX_STAGES;
#ifndef DN_PDL
#define DN_PDL 1  // convolutions launched as programmatic dependents of the kernel before them
#endif
#ifndef DN_TMA_STORE
#define DN_TMA_STORE 1  // folded tiles store their BF16 output with TMA bulk stores
#endif
#ifndef DN_EPI_GROUPS
#define DN_EPI_GROUPS 4
#endif
constexpr int EPI_WARPS = 4;                    // one epilogue warp per TMEM lane quarter
constexpr int EPI_GROUPS = DN_EPI_GROUPS;       // accumulators in flight, one epilogue group each
constexpr int PRODUCER_WARP = EPI_WARPS * EPI_GROUPS;
constexpr int MMA_WARP = PRODUCER_WARP + 1;
constexpr int THREADS = 32 * (MMA_WARP + 1);
// mbarrier slots after the 2 x MAX_STAGES stage barriers
constexpr int BAR_TFULL = 2 * MAX_STAGES, BAR_TEMPTY = BAR_TFULL + EPI_GROUPS, BAR_TMEM = BAR_TEMPTY + EPI_GROUPS,
              BAR_W = BAR_TMEM + 1, BAR_COUNT = BAR_W + 1;
constexpr size_t kFixed = 1024 + 8 * BAR_COUNT + 16 + 1024;  // alignment slack, barriers, bias (256 floats)
constexpr unsigned long long kWaitNs = 2000000000ull;
#ifndef DN_FOLD
#define DN_FOLD 1
#endif
#ifndef DN_C32
#define DN_C32 1
#endif

__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
// Wait for the phase of parity `parity` to complete; false if the bound ran out. The clock
// is read only once the first test has failed.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (!mbar_try(bar, parity))
        if (globaltimer() - t0 > kWaitNs) return false;
    return true;
}

__device__ __forceinline__ void tma_4d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                       unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
// Programmatic dependent launch (griddep_wait / griddep_launch, dn_net.hpp): a convolution's
// prologue (barriers, TMEM, bias, resident weights: data no kernel of the chain writes) runs
// while the kernel before it drains; its producer waits before the first activation load.

// Bulk tensor store of a shared-memory box (bulk-group completion); the box's coordinates
// outside the tensor are not written.
__device__ __forceinline__ void tma_store_4d(const CUtensorMap *map, unsigned src, int c0, int c1, int c2, int c3) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];\n" ::"l"(
                     reinterpret_cast<unsigned long long>(map)),
                 "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(src)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
// Named barrier of `threads` threads that also returns whether `pred` held for all of them.
__device__ __forceinline__ bool bar_and(int id, int threads, bool pred) {
    int r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((int)pred), "r"(id), "r"(threads)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void tma_2d(unsigned dst, const CUtensorMap *map, int c0, int c1, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ unsigned long long sdesc(unsigned addr) {
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) |  // start address
           (1ull << 16) |                                  // leading byte offset (unused here)
           ((unsigned long long)(1024 >> 4) << 32) |       // stride byte offset
           (1ull << 46) |                                  // descriptor version
           (2ull << 61);                                   // 128-byte swizzle
}

// Shared-memory matrix descriptor: K-major, 64-byte swizzle (rows of 32 BF16 channels),
// 8-row groups 512 bytes apart.
__device__ __forceinline__ unsigned long long sdesc64(unsigned addr) {
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((unsigned long long)(512 >> 4) << 32) |
           (1ull << 46) | (4ull << 61);
}

// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D, M = 128, N.
__device__ __forceinline__ unsigned idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(TM >> 4) << 24);
}

__device__ __forceinline__ void umma(unsigned tmem, unsigned long long a, unsigned long long b, unsigned id,
                                     unsigned acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void umma_commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

struct ConvTiles {
    int H, W, Wb, Hb, tx, ty;  // tiles of Wb x Hb pixels, tx x ty per image
    int seg0, cpt;             // 64-channel chunks per tap: of input 0, in total
    int c0, c1;                // channels of input 0 and input 1
    int Cout, N, nhalf, mtiles, ntiles, stages;
    int groups;                // accumulators in flight (groups x nhalf TMEM columns)
    int wres;                  // row tiles: the weights stay resident in shared memory
    int narrow0, narrow1;      // row tiles: input 0 / 1 read as 32-channel rows (64-byte swizzle)
    unsigned astage;           // row tiles: bytes of a stage's row box
    const float *bias;
    int relu;
    bf16 *out_bf;
    float *out_f;
    const float *fin_feat;  // the finished output layer (FOut)
    float *fin_out;
    int fin_H, fin_W;
    int tstore;     // folded tiles: the output goes out through shared memory and TMA stores
                    // (1: BF16 out_bf, 2: FP32 out_f)
    unsigned obuf;  // bytes of an epilogue group's output buffer (FOLD_OUT pixels x Cout)
};

// K steps of 16 that chunk j actually holds: the MMAs over a chunk's zero-filled channels
// (and the matching zero weights) are skipped.
__device__ __forceinline__ int chunk_ksteps(const ConvTiles &q, int j) {
    const int rem = j < q.seg0 ? q.c0 - KB * j : q.c1 - KB * (j - q.seg0);
    return min(KB / 16, (rem + 15) / 16);
}

__device__ __forceinline__ void tmem_ld16(unsigned addr, unsigned (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(addr));
}

// 16 output channels [cb, cb + 16) of pixel p: bias (from shared memory when sbias is given:
// N entries, zero past Cout), ReLU, BF16 and/or FP32 store (channels past Cout are dropped);
// XO: instead of the stores, channels 0..2 finished into the denoised image (FOut).
// Every array index is static, so the values stay in registers.
template <bool XO>
__device__ __forceinline__ void store16(const ConvTiles &q, const unsigned (&v)[16], int cb, long p,
                                        const float *sbias = nullptr) {
    const int Cout = q.Cout;
    float f[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float x_ = __uint_as_float(v[j]);
        if (sbias)
            x_ += sbias[cb + j];
        else if (q.bias)
            x_ += __ldg(q.bias + min(cb + j, Cout - 1));
        if (q.relu) x_ = fmaxf(x_, 0.0f);
        f[j] = x_;
    }
    if (cb + 16 <= Cout) {
        if (q.out_bf) {
            __nv_bfloat162 h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[j] = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
            uint4 *dst = reinterpret_cast<uint4 *>(q.out_bf + p * Cout + cb);
            dst[0] = *reinterpret_cast<uint4 *>(&h[0]);
            dst[1] = *reinterpret_cast<uint4 *>(&h[4]);
        }
        if (!XO && q.out_f) {
            float4 *dst = reinterpret_cast<float4 *>(q.out_f + p * Cout + cb);
#pragma unroll
            for (int j = 0; j < 4; ++j) dst[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
        }
        if (XO && cb == 0) {
            const long x = p % q.W, r = p / q.W;
            const long y = r % q.H, b = r / q.H;
            if (x < q.fin_W && y < q.fin_H) {
                const long o = (b * q.fin_H + y) * q.fin_W + x;
                const float *in = q.fin_feat + o * DN_FEATURES;
                float *dst = q.fin_out + o * 3;
                dst[0] = dn_output(__ldg(in), f[0]);
                dst[1] = dn_output(__ldg(in + 1), f[1]);
                dst[2] = dn_output(__ldg(in + 2), f[2]);
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (cb + j < Cout) {
                if (q.out_bf) q.out_bf[p * Cout + cb + j] = __float2bfloat16_rn(f[j]);
                if (q.out_f) q.out_f[p * Cout + cb + j] = f[j];
            }
    }
}

// Epilogue: group g (warps 4g..4g+3) reads the tiles of accumulator g (every groups-th tile);
// its warp of lane quarter i reads TMEM lanes 32i..32i+31 (tile rows = pixels 32i..32i+31
// of the Wb x Hb block) 32 columns at a time, and hands the accumulator back to the MMA
// thread as soon as its last columns are in registers, before the bias, ReLU and NHWC
// stores of those. Several groups keep several tiles' stores in flight on each SM
// sub-partition. False if a wait gave up.
// 16 output channels [cb, cb + 16) of a pixel into shared memory at `dst` (BF16, bias from
// shared memory, ReLU; channels past Cout dropped), for the group's TMA store.
__device__ __forceinline__ void store16_smem(const ConvTiles &q, const unsigned (&v)[16], int cb, unsigned dst,
                                             const float *sbias) {
    unsigned h[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float a = __uint_as_float(v[2 * j]) + sbias[cb + 2 * j], b = __uint_as_float(v[2 * j + 1]) + sbias[cb + 2 * j + 1];
        if (q.relu) {
            a = fmaxf(a, 0.0f);
            b = fmaxf(b, 0.0f);
        }
        const __nv_bfloat162 t = __floats2bfloat162_rn(a, b);
        h[j] = *reinterpret_cast<const unsigned *>(&t);
    }
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(dst), "r"(h[0]), "r"(h[1]), "r"(h[2]), "r"(h[3])
                 : "memory");
    if (cb + 16 <= q.Cout)  // Cout is a multiple of 8: the last group may hold 8 channels
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(dst + 16u), "r"(h[4]), "r"(h[5]), "r"(h[6]),
                     "r"(h[7])
                     : "memory");
}

// The same for an FP32 output: 16 floats, channels past Cout dropped.
__device__ __forceinline__ void store16_smem_f32(const ConvTiles &q, const unsigned (&v)[16], int cb, unsigned dst,
                                                 const float *sbias) {
    float f[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        f[j] = __uint_as_float(v[j]) + sbias[cb + j];
        if (q.relu) f[j] = fmaxf(f[j], 0.0f);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (cb + 4 * k < q.Cout)
            asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(dst + 16u * k), "f"(f[4 * k]),
                         "f"(f[4 * k + 1]), "f"(f[4 * k + 2]), "f"(f[4 * k + 3])
                         : "memory");
}

template <bool XO, class Origin>
__device__ __forceinline__ bool epilogue(const ConvTiles &q, unsigned tmem, unsigned bar0, int my_tiles,
                                         const Origin &tile_origin) {
    const int warp = threadIdx.x >> 5, g = warp / EPI_WARPS, quarter = warp % EPI_WARPS;
    if (g >= q.groups) return true;
    const int row = (int)threadIdx.x & (TM - 1);  // = 32 quarter + lane
    const int xl = row % q.Wb, yl = row / q.Wb;
    const unsigned tfull = bar0 + 8u * (BAR_TFULL + g), tempty = bar0 + 8u * (BAR_TEMPTY + g);
    unsigned use = 0;
    for (int lt = g; lt < my_tiles; lt += q.groups, ++use) {
        if (!__all_sync(0xffffffffu, mbar_wait(tfull, use & 1u))) return false;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        int x0, y0, n, n0;
        tile_origin((int)blockIdx.x + lt * (int)gridDim.x, x0, y0, n, n0);
        const int x = x0 + xl, y = y0 + yl;
        const bool inside = x < q.W && y < q.H;
        const long p = ((long)n * q.H + y) * q.W + x;
        const unsigned taddr = tmem + ((unsigned)(32 * quarter) << 16) + (unsigned)(g * q.nhalf);
        for (int c0 = 0; c0 < q.N; c0 += 32) {
            const bool two = c0 + 16 < q.N;
            unsigned va[16], vb[16];
            tmem_ld16(taddr + c0, va);
            if (two) tmem_ld16(taddr + c0 + 16, vb);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (c0 + 32 >= q.N) {  // the accumulator is free for the MMAs again
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
                mbar_arrive(tempty);
            }
            const int cb = n0 + c0;
            if (inside && cb < q.Cout) {
                store16<XO>(q, va, cb, p);
                if (two && cb + 16 < q.Cout) store16<XO>(q, vb, cb + 16, p);
            }
        }
    }
    return true;
}

template <bool XO>
__global__ void __launch_bounds__(THREADS, 1)
    k_conv_umma(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                const __grid_constant__ CUtensorMap tmw, const ConvTiles q) {
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = saddr(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;
    const unsigned a_bytes = TM * 128, stage_bytes = a_bytes + (unsigned)q.N * 128;
    const int S = q.stages;
    const unsigned bar0 = base + S * stage_bytes;
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 8u * (MAX_STAGES + st); };
    auto tfull = [&](int a) { return bar0 + 8u * (BAR_TFULL + a); };
    auto tempty = [&](int a) { return bar0 + 8u * (BAR_TEMPTY + a); };
    const unsigned tmem_slot = bar0 + 8u * BAR_TMEM;
    const unsigned *tmem_slot_ptr = reinterpret_cast<const unsigned *>(smem_raw + (tmem_slot - raw));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int KT = 9 * q.cpt;
    const int my_tiles = q.ntiles > (int)blockIdx.x ? (q.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    // Tile t: output channels [N (t / mtiles), +N) of the pixel block t % mtiles.
    auto tile_origin = [&](int t, int &x0, int &y0, int &n, int &n0) {
        const int mt = t % q.mtiles;
        n0 = (t / q.mtiles) * q.N;
        x0 = (mt % q.tx) * q.Wb;
        const int r = mt / q.tx;
        y0 = (r % q.ty) * q.Hb;
        n = r / q.ty;
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tmem_slot),
                     "r"(q.groups * q.nhalf));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 1);
        }
        for (int a = 0; a < EPI_GROUPS; ++a) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), 32 * EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = *tmem_slot_ptr;
    bool ok = true;

    griddep_launch();
    if (warp == PRODUCER_WARP) {
        // ---- TMA producer: one thread. Stage index and phase advance incrementally (this
        // thread's issue rate bounds the pipeline: no divisions in the loop).
        if (lane == 0) {
            griddep_wait();
            const unsigned tx_bytes = a_bytes + (unsigned)q.N * 128;
            int st = 0;
            unsigned ph = 0;     // parity of the current use of stage st
            bool refill = false;  // every stage has been used once: wait for its MMAs first
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                int x0, y0, n, n0;
                tile_origin((int)blockIdx.x + lt * (int)gridDim.x, x0, y0, n, n0);
                int kcoord = 0;
                for (int tap = 0; tap < 9 && ok; ++tap) {
                    const int dy = tap / 3 - 1, dx = tap - 3 * (dy + 1) - 1;
                    for (int j = 0; j < q.cpt; ++j, kcoord += KB) {
                        if (refill && !(ok = mbar_wait(empty(st), ph ^ 1u))) break;
                        const unsigned sa = base + st * stage_bytes;
                        mbar_expect_tx(full(st), tx_bytes);
                        if (j < q.seg0)
                            tma_4d(sa, &tm0, j * KB, x0 + dx, y0 + dy, n, full(st));
                        else
                            tma_4d(sa, &tm1, (j - q.seg0) * KB, x0 + dx, y0 + dy, n, full(st));
                        tma_2d(sa + a_bytes, &tmw, kcoord, n0, full(st));
                        if (++st == S) {
                            st = 0;
                            ph ^= 1u;
                            refill = true;
                        }
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == MMA_WARP) {
        // ---- MMA issue: one thread.
        if (lane == 0) {
            const unsigned id = idesc(q.N);
            int st = 0;
            unsigned ph = 0;
            int a = 0;         // accumulator of tile lt
            unsigned use = 0;  // earlier tiles in accumulator a
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                if (use > 0 && !(ok = mbar_wait(tempty(a), (use - 1) & 1u))) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const unsigned d = tmem + (unsigned)(a * q.nhalf);
                unsigned acc = 0;
                for (int kb = 0, j = 0; kb < KT; ++kb) {
                    if (!(ok = mbar_wait(full(st), ph))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                    const unsigned sa = base + st * stage_bytes, sb = sa + a_bytes;
                    const int ks = chunk_ksteps(q, j);
                    for (int kk = 0; kk < ks; ++kk) {
                        umma(d, sdesc(sa + 32 * kk), sdesc(sb + 32 * kk), id, acc);
                        acc = 1;
                    }
                    umma_commit(empty(st));
                    if (++st == S) {
                        st = 0;
                        ph ^= 1u;
                    }
                    if (++j == q.cpt) j = 0;
                }
                if (ok) umma_commit(tfull(a));
                if (++a == q.groups) {
                    a = 0;
                    ++use;
                }
            }
        }
        __syncwarp();
    } else {
        ok = epilogue<XO>(q, tmem, bar0, my_tiles, tile_origin);
    }
    if (!ok) atomicOr(&g_umma_status, 1u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(q.groups * q.nhalf));
    }
}

// Row tiles (Wb = 128, Hb = 1: every tile is 128 pixels of one image row). The three
// horizontal taps of one kernel row read the same pixels shifted by one, so one TMA box of
// 130 pixels x 64 channels at (x0 - 1, y0 + dy) serves all three: the A operand of tap dx
// (-1, 0, 1) starts dx + 1 rows of 128 bytes into the box. Per tile and 64-channel chunk
// that is three boxes instead of nine. The 128-byte swizzle is a function of the
// shared-memory address (bits 4-6 XOR bits 7-9, as TMA writes it), so a descriptor that
// starts one or two rows into the box reads the shifted rows correctly with its base-offset
// field left at 0 (measured: the parity tests fail when that field carries the row phase).
// When every k-block of the packed weights fits in shared memory beside the pipeline (one
// output-channel tile), the weights are loaded once per CTA and stay resident; otherwise
// each stage also carries the three k-blocks of its taps.
constexpr int HALO = TM + 2;                  // pixels of a row box
constexpr unsigned HALO_BYTES = HALO * 128;   // bytes of a row box of 64 channels (16,640)
constexpr unsigned HALO_STAGE = 17 * 1024;    // ... rounded up to the 1024-byte swizzle period
constexpr unsigned HALO32_BYTES = HALO * 64;  // bytes of a row box of 32 channels (8,320)
constexpr unsigned HALO32_STAGE = 9 * 1024;

// Three taps (dx = -1, 0, 1) of one row box: KS K steps of 16 each. The descriptors' address
// field counts 16-byte units: a K step is 32 bytes (+2), a row is rstep units.
template <int KS>
__device__ __forceinline__ void mma_taps(unsigned d, unsigned long long ad, const unsigned long long (&bd)[3],
                                         unsigned rstep, unsigned id, unsigned &acc) {
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int kk = 0; kk < KS; ++kk) {
            umma(d, ad + dx * rstep + 2 * kk, bd[dx] + 2 * kk, id, acc);
            acc = 1;
        }
}


template <bool XO>
__global__ void __launch_bounds__(THREADS, 1)
    k_conv_rows(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                const __grid_constant__ CUtensorMap tmw, const ConvTiles q) {
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = saddr(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;
    const unsigned kblk = (unsigned)q.N * 128;  // one k-block of weights: N rows x 64 K
    const int KT = 9 * q.cpt;
    const unsigned wbytes = q.wres ? (unsigned)KT * kblk : 0u;
    const unsigned stage_bytes = q.astage + (q.wres ? 0u : 3u * kblk);
    const int S = q.stages;
    const unsigned sbase = base + wbytes;
    const unsigned bar0 = sbase + S * stage_bytes;
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 8u * (MAX_STAGES + st); };
    auto tfull = [&](int a) { return bar0 + 8u * (BAR_TFULL + a); };
    auto tempty = [&](int a) { return bar0 + 8u * (BAR_TEMPTY + a); };
    const unsigned tmem_slot = bar0 + 8u * BAR_TMEM;
    const unsigned wfull = bar0 + 8u * BAR_W;
    const unsigned *tmem_slot_ptr = reinterpret_cast<const unsigned *>(smem_raw + (tmem_slot - raw));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int my_tiles = q.ntiles > (int)blockIdx.x ? (q.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_origin = [&](int t, int &x0, int &y0, int &n, int &n0) {
        const int mt = t % q.mtiles;
        n0 = (t / q.mtiles) * q.N;
        x0 = (mt % q.tx) * TM;
        const int r = mt / q.tx;
        y0 = r % q.ty;
        n = r / q.ty;
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tmem_slot),
                     "r"(q.groups * q.nhalf));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 1);
        }
        for (int a = 0; a < EPI_GROUPS; ++a) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), 32 * EPI_WARPS);
        }
        mbar_init(wfull, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = *tmem_slot_ptr;
    bool ok = true;

    griddep_launch();
    if (warp == PRODUCER_WARP) {
        // ---- TMA producer: one thread.
        if (lane == 0) {
            if (q.wres && my_tiles > 0) {
                mbar_expect_tx(wfull, wbytes);
                for (int kb = 0; kb < KT; ++kb) tma_2d(base + kb * kblk, &tmw, kb * KB, 0, wfull);
            }
            griddep_wait();
            const unsigned wtx = q.wres ? 0u : 3u * kblk;
            int st = 0;
            unsigned ph = 0;
            bool refill = false;
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                int x0, y0, n, n0;
                tile_origin((int)blockIdx.x + lt * (int)gridDim.x, x0, y0, n, n0);
                for (int j = 0; j < q.cpt && ok; ++j) {
                    const bool in0 = j < q.seg0;
                    const bool narrow = in0 ? q.narrow0 : q.narrow1;
                    const unsigned tx_bytes = (narrow ? HALO32_BYTES : HALO_BYTES) + wtx;
                    for (int dy = -1; dy <= 1; ++dy) {
                        if (refill && !(ok = mbar_wait(empty(st), ph ^ 1u))) break;
                        const unsigned sa = sbase + st * stage_bytes;
                        mbar_expect_tx(full(st), tx_bytes);
                        if (in0)
                            tma_4d(sa, &tm0, j * KB, x0 - 1, y0 + dy, n, full(st));
                        else
                            tma_4d(sa, &tm1, (j - q.seg0) * KB, x0 - 1, y0 + dy, n, full(st));
                        if (!q.wres)
                            for (int dx = 0; dx < 3; ++dx)
                                tma_2d(sa + q.astage + dx * kblk, &tmw, (((dy + 1) * 3 + dx) * q.cpt + j) * KB, n0,
                                       full(st));
                        if (++st == S) {
                            st = 0;
                            ph ^= 1u;
                            refill = true;
                        }
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == MMA_WARP) {
        // ---- MMA issue: one thread; three taps per stage.
        if (lane == 0) {
            const unsigned id = idesc(q.N);
            if (q.wres && my_tiles > 0) ok = mbar_wait(wfull, 0);
            int st = 0;
            unsigned ph = 0;
            int a = 0;         // accumulator of tile lt
            unsigned use = 0;  // earlier tiles in accumulator a
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                if (use > 0 && !(ok = mbar_wait(tempty(a), (use - 1) & 1u))) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const unsigned d = tmem + (unsigned)(a * q.nhalf);
                unsigned acc = 0;
                for (int j = 0; j < q.cpt && ok; ++j) {
                    const bool narrow = j < q.seg0 ? q.narrow0 : q.narrow1;
                    const int ks = chunk_ksteps(q, j);
                    for (int dy = 0; dy < 3; ++dy) {
                        if (!(ok = mbar_wait(full(st), ph))) break;
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                        const unsigned sa = sbase + st * stage_bytes;
                        const unsigned long long ad = narrow ? sdesc64(sa) : sdesc(sa);
                        const unsigned rstep = narrow ? 4u : 8u;
                        unsigned long long bd[3];
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx)
                            bd[dx] = sdesc(q.wres ? base + (unsigned)((dy * 3 + dx) * q.cpt + j) * kblk
                                                  : sa + q.astage + dx * kblk);
                        switch (ks) {
                            case 1: mma_taps<1>(d, ad, bd, rstep, id, acc); break;
                            case 2: mma_taps<2>(d, ad, bd, rstep, id, acc); break;
                            case 3: mma_taps<3>(d, ad, bd, rstep, id, acc); break;
                            default: mma_taps<4>(d, ad, bd, rstep, id, acc); break;
                        }
                        umma_commit(empty(st));
                        if (++st == S) {
                            st = 0;
                            ph ^= 1u;
                        }
                    }
                }
                if (ok) umma_commit(tfull(a));
                if (++a == q.groups) {
                    a = 0;
                    ++use;
                }
            }
        }
        __syncwarp();
    } else {
        ok = epilogue<XO>(q, tmem, bar0, my_tiles, tile_origin);
    }
    if (!ok) atomicOr(&g_umma_status, 1u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(q.groups * q.nhalf));
    }
}

// Folded row tiles. The three horizontal taps go into N instead of into three MMAs: with
// A = 128 input pixels and B = the weights of taps (dy, -1), (dy, 0), (dy, +1) stacked as
// 3 N rows, D[r][(b, co)] is tap dx = b - 1's contribution of input pixel r. The output at
// pixel r sums D[r - 1][(0, co)], D[r][(1, co)] and D[r + 1][(2, co)] over dy and the
// chunks, and the epilogue gathers the neighbours' columns with warp shuffles. So that no
// neighbour lies in another warp, lane quarter i (A rows 32i..32i+31) holds input pixels
// x0 - 1 + 30i + (0..31) and outputs its lanes 1..30: a tile yields 120 outputs (the widths
// of a 1920-pixel pyramid are multiples of 120) and reads four 32-pixel boxes per row.
// One stage holds the three rows (dy) of one chunk and is released by one commit: per tile
// cpt x 3 x K-steps MMAs of N = 3 Cout and cpt + 1 commits (6 MMAs and 2 commits for
// 32 -> 32 channels, against 18 MMAs of N = 32 and 4 commits unfolded). The weights are
// resident, laid out [dy][chunk][dx][N rows].
constexpr int FOLD_OUT = 120;               // outputs per folded tile
constexpr int FOLD_STEP = 30;               // outputs per lane quarter
constexpr unsigned ROW_BOX = TM * 128;      // 128 rows of 64 channels (16 KB)
constexpr unsigned ROW32_BOX = TM * 64;     // 128 rows of 32 channels (8 KB)

template <int KS>
__device__ __forceinline__ void mma_rows3(unsigned d, unsigned long long ad, unsigned abox16,
                                          const unsigned long long (&bd)[3], unsigned id, unsigned &acc) {
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int kk = 0; kk < KS; ++kk) {
            umma(d, ad + dy * abox16 + 2 * kk, bd[dy] + 2 * kk, id, acc);
            acc = 1;
        }
}

// Epilogue of the folded tiles: group g reads accumulator g, 16 output channels at a time
// (columns c0, N + c0, 2N + c0), adds each row's neighbours' columns and stores lanes 1..30.
// With q.tstore (BF16 or FP32 output, XO false) the group's four warps write the tile into their
// shared-memory buffer `obuf0 + g * q.obuf` ([pixel][channel], FOLD_OUT pixels) and one
// thread stores it with a TMA bulk store; the group's named barrier (id 1 + g) orders the
// buffer's reuse, and every warp of the group takes the same exits.
template <bool XO, class Origin>
__device__ __forceinline__ bool epilogue_fold(const ConvTiles &q, unsigned tmem, unsigned bar0, const float *sbias,
                                              int my_tiles, const Origin &tile_origin, const CUtensorMap *tmo,
                                              unsigned obuf0) {
    const int warp = threadIdx.x >> 5, g = warp / EPI_WARPS, quarter = warp % EPI_WARPS;
    const int lane = threadIdx.x & 31;
    if (g >= q.groups) return true;
    const unsigned tfull = bar0 + 8u * (BAR_TFULL + g), tempty = bar0 + 8u * (BAR_TEMPTY + g);
    const bool ts = !XO && q.tstore;
    const bool leader = quarter == 0 && lane == 0;
    const unsigned ob = obuf0 + (unsigned)g * q.obuf;
    unsigned use = 0;
    for (int lt = g; lt < my_tiles; lt += q.groups, ++use) {
        const bool okw = __all_sync(0xffffffffu, mbar_wait(tfull, use & 1u));
        if (ts) {
            // The buffer is free once the previous bulk store has read it.
            if (leader) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
            if (!bar_and(1 + g, 32 * EPI_WARPS, okw)) {
                if (leader) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
                return false;
            }
        } else if (!okw) {
            return false;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        int x0, y0, n, n0;
        tile_origin((int)blockIdx.x + lt * (int)gridDim.x, x0, y0, n, n0);
        const int x = x0 - 1 + FOLD_STEP * quarter + lane;
        const bool store = lane >= 1 && lane <= FOLD_STEP && x < q.W;
        const long p = ((long)n * q.H + y0) * q.W + x;
        const unsigned esz = q.tstore == 2 ? 4u : 2u;
        const unsigned orow = ob + (unsigned)((x - x0) * q.Cout) * esz;  // this pixel's row of the buffer
        const unsigned taddr = tmem + ((unsigned)(32 * quarter) << 16) + (unsigned)(g * q.nhalf);
        for (int c0 = 0; c0 < q.N; c0 += 16) {
            unsigned b0[16], b1[16], b2[16];
            tmem_ld16(taddr + c0, b0);
            tmem_ld16(taddr + q.N + c0, b1);
            tmem_ld16(taddr + 2 * q.N + c0, b2);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (c0 + 16 >= q.N) {  // the accumulator is free for the MMAs again
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
                mbar_arrive(tempty);
            }
            unsigned v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float up = __shfl_up_sync(0xffffffffu, __uint_as_float(b0[j]), 1);
                const float dn = __shfl_down_sync(0xffffffffu, __uint_as_float(b2[j]), 1);
                v[j] = __float_as_uint(up + __uint_as_float(b1[j]) + dn);
            }
            const int cb = n0 + c0;
            if (store && cb < q.Cout) {
                if (ts && q.tstore == 2) store16_smem_f32(q, v, cb, orow + (unsigned)cb * 4u, sbias);
                else if (ts) store16_smem(q, v, cb, orow + (unsigned)cb * 2u, sbias);
                else store16<XO>(q, v, cb, p, sbias);
            }
        }
        if (ts) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            bar_and(1 + g, 32 * EPI_WARPS, true);
            if (leader) tma_store_4d(tmo, ob, 0, x0, y0, n);
        }
    }
    if (ts && leader) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    return true;
}

template <bool XO>
__global__ void __launch_bounds__(THREADS, 1)
    k_conv_fold(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                const __grid_constant__ CUtensorMap tmw, const __grid_constant__ CUtensorMap tmo, const ConvTiles q) {
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = saddr(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;
    const unsigned kblk = (unsigned)q.N * 128;
    const int KT = 9 * q.cpt;
    const unsigned wbytes = (unsigned)KT * kblk;
    const unsigned stage_bytes = q.astage;  // three row boxes
    const int S = q.stages;
    const unsigned sbase = base + wbytes;
    const unsigned bar0 = sbase + S * stage_bytes;
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 8u * (MAX_STAGES + st); };
    auto tfull = [&](int a) { return bar0 + 8u * (BAR_TFULL + a); };
    auto tempty = [&](int a) { return bar0 + 8u * (BAR_TEMPTY + a); };
    const unsigned tmem_slot = bar0 + 8u * BAR_TMEM;
    const unsigned wfull = bar0 + 8u * BAR_W;
    const unsigned *tmem_slot_ptr = reinterpret_cast<const unsigned *>(smem_raw + (tmem_slot - raw));
    float *sbias = reinterpret_cast<float *>(smem_raw + (bar0 + 8u * BAR_COUNT - raw));  // N floats
    // the epilogue groups' output buffers (q.tstore), 128-byte aligned after the bias
    const unsigned obuf0 = (bar0 + 8u * BAR_COUNT + 1024u + 127u) & ~127u;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int my_tiles = q.ntiles > (int)blockIdx.x ? (q.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_origin = [&](int t, int &x0, int &y0, int &n, int &n0) {
        const int mt = t % q.mtiles;
        n0 = 0;
        x0 = (mt % q.tx) * FOLD_OUT;
        const int r = mt / q.tx;
        y0 = r % q.ty;
        n = r / q.ty;
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tmem_slot),
                     "r"(q.groups * q.nhalf));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 1);
        }
        for (int a = 0; a < EPI_GROUPS; ++a) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), 32 * EPI_WARPS);
        }
        mbar_init(wfull, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    for (int c = tid; c < q.N; c += THREADS) sbias[c] = (q.bias && c < q.Cout) ? q.bias[c] : 0.0f;
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = *tmem_slot_ptr;
    bool ok = true;

    griddep_launch();
    if (warp == PRODUCER_WARP) {
        if (lane == 0) {
            if (my_tiles > 0) {
                // packed k-block (tap, j) -> resident slot [dy][j][dx]
                mbar_expect_tx(wfull, wbytes);
                for (int kb = 0; kb < KT; ++kb) {
                    const int tap = kb / q.cpt, j = kb - tap * q.cpt, dy = tap / 3, dx = tap - 3 * dy;
                    tma_2d(base + (unsigned)((dy * q.cpt + j) * 3 + dx) * kblk, &tmw, kb * KB, 0, wfull);
                }
            }
            griddep_wait();
            int st = 0;
            unsigned ph = 0;
            bool refill = false;
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                int x0, y0, n, n0;
                tile_origin((int)blockIdx.x + lt * (int)gridDim.x, x0, y0, n, n0);
                for (int j = 0; j < q.cpt; ++j) {
                    if (refill && !(ok = mbar_wait(empty(st), ph ^ 1u))) break;
                    const bool in0 = j < q.seg0;
                    const unsigned box = (in0 ? q.narrow0 : q.narrow1) ? ROW32_BOX : ROW_BOX;
                    const unsigned sa = sbase + st * stage_bytes;
                    mbar_expect_tx(full(st), 3 * box);
                    for (int dy = 0; dy < 3; ++dy)
                        for (int i = 0; i < EPI_WARPS; ++i) {  // 32-pixel boxes, 30 apart
                            const unsigned dst = sa + dy * box + i * (box / EPI_WARPS);
                            const int xi = x0 - 1 + FOLD_STEP * i;
                            if (in0)
                                tma_4d(dst, &tm0, j * KB, xi, y0 + dy - 1, n, full(st));
                            else
                                tma_4d(dst, &tm1, (j - q.seg0) * KB, xi, y0 + dy - 1, n, full(st));
                        }
                    if (++st == S) {
                        st = 0;
                        ph ^= 1u;
                        refill = true;
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            const unsigned id = idesc(3 * q.N);
            if (my_tiles > 0) ok = mbar_wait(wfull, 0);
            int st = 0;
            unsigned ph = 0;
            int a = 0;
            unsigned use = 0;
            for (int lt = 0; lt < my_tiles && ok; ++lt) {
                if (use > 0 && !(ok = mbar_wait(tempty(a), (use - 1) & 1u))) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const unsigned d = tmem + (unsigned)(a * q.nhalf);
                unsigned acc = 0;
                for (int j = 0; j < q.cpt; ++j) {
                    if (!(ok = mbar_wait(full(st), ph))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                    const bool narrow = j < q.seg0 ? q.narrow0 : q.narrow1;
                    const unsigned sa = sbase + st * stage_bytes;
                    const unsigned long long ad = narrow ? sdesc64(sa) : sdesc(sa);
                    const unsigned abox16 = (narrow ? ROW32_BOX : ROW_BOX) >> 4;
                    unsigned long long bd[3];
#pragma unroll
                    for (int dy = 0; dy < 3; ++dy) bd[dy] = sdesc(base + (unsigned)((dy * q.cpt + j) * 3) * kblk);
                    switch (chunk_ksteps(q, j)) {
                        case 1: mma_rows3<1>(d, ad, abox16, bd, id, acc); break;
                        case 2: mma_rows3<2>(d, ad, abox16, bd, id, acc); break;
                        case 3: mma_rows3<3>(d, ad, abox16, bd, id, acc); break;
                        default: mma_rows3<4>(d, ad, abox16, bd, id, acc); break;
                    }
                    umma_commit(empty(st));
                    if (++st == S) {
                        st = 0;
                        ph ^= 1u;
                    }
                }
                if (ok) umma_commit(tfull(a));
                if (++a == q.groups) {
                    a = 0;
                    ++use;
                }
            }
        }
        __syncwarp();
    } else {
        ok = epilogue_fold<XO>(q, tmem, bar0, sbias, my_tiles, tile_origin, &tmo, obuf0);
    }
    if (!ok) atomicOr(&g_umma_status, 1u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(q.groups * q.nhalf));
    }
}

// Nearest 2x upsampling, NHWC: y (B, 2h, 2w, C) from x (B, h, w, C); a thread copies 8
// channels of one input pixel to its 2 x 2 output pixels.
__global__ void k_upsample2(const bf16 *__restrict__ x, int B, int h, int w, int C, bf16 *__restrict__ y) {
    griddep_wait();  // a programmatic dependent of the kernel that wrote x
    griddep_launch();
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int c8 = C / 8;
    const size_t n = (size_t)B * h * w * c8;
    if (i >= n) return;
    const int c = (int)(i % c8) * 8;
    size_t r = i / c8;
    const int xx = (int)(r % w);
    r /= w;
    const int yy = (int)(r % h);
    const int b = (int)(r / h);
    const uint4 v = *reinterpret_cast<const uint4 *>(x + (i / c8) * C + c);
    bf16 *o = y + (((size_t)b * 2 * h + 2 * yy) * 2 * w + 2 * xx) * C + c;
    const size_t row = (size_t)2 * w * C;
    *reinterpret_cast<uint4 *>(o) = v;
    *reinterpret_cast<uint4 *>(o + C) = v;
    *reinterpret_cast<uint4 *>(o + row) = v;
    *reinterpret_cast<uint4 *>(o + row + C) = v;
}

// Forward packing: wpk[co][(tap cpt + j) 64 + cc] = w[tap][ci][co] for the input channel ci
// of chunk j (chunks of input 0 first, then of input 1), zero past either channel count.
template <class T>
__device__ __forceinline__ float pack_fwd_value(const T *w, int c0, int c1, int cout, size_t idx) {
    const int seg0 = (c0 + 63) / 64, cpt = seg0 + (c1 + 63) / 64;
    const size_t kp = (size_t)9 * cpt * 64;
    const int co = (int)(idx / kp);
    const int k = (int)(idx % kp);
    const int kb = k / 64, cc = k % 64;
    const int tap = kb / cpt, j = kb % cpt;
    int ci;
    if (j < seg0) {
        ci = j * 64 + cc;
        if (ci >= c0) return 0.0f;
    } else {
        const int c = (j - seg0) * 64 + cc;
        if (c >= c1) return 0.0f;
        ci = c0 + c;
    }
    return (float)w[((size_t)tap * (c0 + c1) + ci) * cout + co];
}

// Data-gradient packing: wpkd[ci][(tap' cptd + j) 64 + cc] = w[8 - tap'][ci][co = 64 j + cc].
__device__ __forceinline__ float pack_bwd_value(const float *w, int cin, int cout, size_t idx) {
    const int cptd = (cout + 63) / 64;
    const size_t kp = (size_t)9 * cptd * 64;
    const int ci = (int)(idx / kp);
    const int k = (int)(idx % kp);
    const int kb = k / 64, cc = k % 64;
    const int tap = kb / cptd, co = (kb % cptd) * 64 + cc;
    if (co >= cout) return 0.0f;
    return w[((size_t)(8 - tap) * cin + ci) * cout + co];
}

template <class T>
__global__ void k_pack_fwd(const T *__restrict__ w, int c0, int c1, int cout, bf16 *__restrict__ out, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(pack_fwd_value(w, c0, c1, cout, i));
}

__global__ void k_pack_bwd(const float *__restrict__ w, int cin, int cout, bf16 *__restrict__ out, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(pack_bwd_value(w, cin, cout, i));
}

// Every layer's packed forward and data-gradient weights from the FP32 parameters.
__global__ void k_pack_all(const float *__restrict__ params, PackTable tab, bf16 *__restrict__ wk,
                           bf16 *__restrict__ wkd) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < tab.fwd_total) {
        int l = 0;
        while (l + 1 < tab.n && i >= tab.e[l + 1].fwd_off) ++l;
        const PackEntry &e = tab.e[l];
        wk[i] = __float2bfloat16_rn(pack_fwd_value(params + e.woff, (int)e.c0, (int)e.c1, (int)e.cout, i - e.fwd_off));
    } else if (i < tab.fwd_total + tab.bwd_total) {
        const size_t j = i - tab.fwd_total;
        int l = 0;
        while (l + 1 < tab.n && j >= tab.e[l + 1].bwd_off) ++l;
        const PackEntry &e = tab.e[l];
        wkd[j] = __float2bfloat16_rn(pack_bwd_value(params + e.woff, (int)(e.c0 + e.c1), (int)e.cout, j - e.bwd_off));
    }
}

// ---- weight gradient ----------------------------------------------------------------------------
// dw[tap][ci][co] = sum_p x[p + off(tap), ci] g[p, co] on the tensor cores, as implicit GEMMs
//   D[(tap, ci)][co] += sum_p X_tap[p][ci] G[p][co]
// whose K runs over pixels. The input is cut into "atoms" of AW channels (64, or 32 where that
// needs fewer M tiles): a slot is one (tap, atom) pair, and an M tile of 128 rows holds
// 128 / AW consecutive slots. Both operands are TMA boxes of one atom (or of 64 output
// channels) x 64 pixels -- one 128- or 64-byte row per pixel with the matching swizzle --
// which tcgen05.mma reads in the MN-major layout: channels contiguous, 8-pixel row groups
// 1024 (512) bytes apart, atoms one box apart. The box of tap (dy, dx) starts at the tile's
// pixel (x0 + dx, y0 + dy): the copy engine's zero fill outside the image is the
// convolution's zero padding, and pixels of the tile outside the image have G = 0.
// Putting taps and channels into M and the output channels into N makes every MMA 128 x
// Cout x 16: on the GB300 an MMA of these narrow layers costs about the same whatever its
// size, so few wide ones are what pays (9 taps of a 32-channel input: 3 MMAs per 16 pixels).
// Row tiles of 32-channel atoms ("rows3") go further: one box of 68 pixels from x0 - 1 per
// (kernel row, atom) holds the three horizontal taps, and an M tile reads it from pixel rows
// 0, 1, 2 (and an unused 3) as its four 32-row atoms, 64 bytes apart: a third of the boxes.
//
// A CTA owns a group of M tiles (their accumulators, Cout columns each, fill at most 512
// TMEM columns) and a contiguous range of 64-pixel tiles (split K). One thread issues the TMA
// loads into a ring of stages, one thread the MMAs, and the four warps then read the
// accumulators back with tcgen05.ld (warp w: lanes = rows 32w..32w+31) and store FP32 partial
// sums per pixel range, which reduce_chunks adds in a fixed order.
constexpr int WG_KC = 64;                             // pixels per tile (one box)
constexpr unsigned WG_ROWS3_BOX = (WG_KC + 4) * 64;   // rows3: 68 pixels x 32 channels
constexpr unsigned WG_ROWS3_STRIDE = 5 * 1024;        // its slot in a stage (1024-aligned)
constexpr int WG_MAX_STAGES = 8;

struct WgradTiles {
    int B, H, W, Wb, Hb, tx, ty, tiles;  // 64-pixel tiles of Wb x Hb pixels
    int Cout, N, ga;                     // output channels, MMA N (Cout rounded to 16), G atoms
    int c0, c1, aw, seg0, apt;           // inputs, atom width, atoms of input 0, atoms per tap
    int spt, mtiles, mt_per_cta;         // slots per M tile, M tiles, M tiles per CTA
    int rows3;                           // row tiles of 32-channel atoms, one box per kernel row
    int cols, tiles_per_chunk, stages;
    float *partial;                      // [chunk][tap][ci][co]
};

// MN-major shared-memory descriptor: atoms of 64 (128-byte swizzle) or 32 (64-byte swizzle)
// channels x 8 pixel rows; 8-row groups `sbo` apart, atoms `lbo` apart.
__device__ __forceinline__ unsigned long long sdesc_mn(unsigned addr, unsigned lbo, unsigned sbo, bool sw64) {
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)(lbo >> 4) << 16) |
           ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46) | ((sw64 ? 4ull : 2ull) << 61);
}

// kind::f16, BF16 A and B both MN-major, FP32 D, M = 128 x N.
__device__ __forceinline__ unsigned idesc_mn(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((unsigned)(n >> 3) << 17) |
           ((unsigned)(TM >> 4) << 24);
}

__global__ void __launch_bounds__(128, 2)
    k_wgrad_umma(const __grid_constant__ CUtensorMap tmg, const __grid_constant__ CUtensorMap tm0,
                 const __grid_constant__ CUtensorMap tm1, const WgradTiles q) {
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = saddr(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;
    const bool sw64 = q.aw == 32;
    // bytes of one G box and of one X box (rows3: 68 pixels of 32 channels, 5 KB apart)
    const unsigned gbox = WG_KC * 128, xbox = q.rows3 ? WG_ROWS3_STRIDE : WG_KC * 2 * q.aw;
    const unsigned g_bytes = (unsigned)q.ga * gbox;
    const int mt0 = blockIdx.y * q.mt_per_cta;
    const int my_mt = min(q.mt_per_cta, q.mtiles - mt0);
    const int slot0 = mt0 * q.spt, slots = min(my_mt * q.spt, 9 * q.apt - slot0);
    const unsigned stage_bytes = g_bytes + (unsigned)(q.mt_per_cta * (q.rows3 ? 1 : q.spt)) * xbox;
    const int S = q.stages;
    const unsigned bar0 = base + S * stage_bytes;
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 8u * (WG_MAX_STAGES + st); };
    const unsigned done = bar0 + 8u * (2 * WG_MAX_STAGES);
    const unsigned tmem_slot = done + 8u;
    const unsigned *tmem_slot_ptr = reinterpret_cast<const unsigned *>(smem_raw + (tmem_slot - raw));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x;
    const int t_begin = chunk * q.tiles_per_chunk;
    const int t_end = min(q.tiles, t_begin + q.tiles_per_chunk);
    const int my_tiles = max(0, t_end - t_begin);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tmem_slot),
                     "r"(q.cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = *tmem_slot_ptr;
    bool ok = true;

    if (tid == 0 && my_tiles > 0) {
        // TMA producer: per 64-pixel tile, the G boxes and one box per slot of this CTA
        // (rows3: one per M tile)
        const unsigned bytes = g_bytes + (q.rows3 ? (unsigned)my_mt * WG_ROWS3_BOX : (unsigned)slots * xbox);
        for (int k = 0; k < my_tiles && ok; ++k) {
            const int st = k % S;
            if (k >= S && !mbar_wait(empty(st), (unsigned)((k / S - 1) & 1))) {
                ok = false;
                break;
            }
            const int t = t_begin + k;
            const int x0 = (t % q.tx) * q.Wb;
            const int r = t / q.tx;
            const int y0 = (r % q.ty) * q.Hb, n = r / q.ty;
            const unsigned sa = base + st * stage_bytes;
            mbar_expect_tx(full(st), bytes);
            for (int a = 0; a < q.ga; ++a) tma_4d(sa + a * gbox, &tmg, 64 * a, x0, y0, n, full(st));
            if (q.rows3) {
                for (int j = 0; j < my_mt; ++j) {
                    const int i = mt0 + j, dy = i / q.apt - 1, atom = i % q.apt;
                    const unsigned dst = sa + g_bytes + j * xbox;
                    if (atom < q.seg0)
                        tma_4d(dst, &tm0, 32 * atom, x0 - 1, y0 + dy, n, full(st));
                    else
                        tma_4d(dst, &tm1, 32 * (atom - q.seg0), x0 - 1, y0 + dy, n, full(st));
                }
                continue;
            }
            for (int j = 0; j < slots; ++j) {
                const int slot = slot0 + j, tap = slot / q.apt, atom = slot % q.apt;
                const int dy = tap / 3 - 1, dx = tap % 3 - 1;
                const unsigned dst = sa + g_bytes + j * xbox;
                if (atom < q.seg0)
                    tma_4d(dst, &tm0, q.aw * atom, x0 + dx, y0 + dy, n, full(st));
                else
                    tma_4d(dst, &tm1, q.aw * (atom - q.seg0), x0 + dx, y0 + dy, n, full(st));
            }
        }
    } else if (tid == 32 && my_tiles > 0) {
        // MMA issuer: per 16-pixel step one 128 x N MMA per M tile
        const unsigned id = idesc_mn(q.N);
        const unsigned xsbo = sw64 ? 512u : 1024u;
        for (int k = 0; k < my_tiles && ok; ++k) {
            const int st = k % S;
            if (!mbar_wait(full(st), (unsigned)((k / S) & 1))) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const unsigned sa = base + st * stage_bytes;
#pragma unroll 1
            for (int ks = 0; ks < WG_KC / 16; ++ks) {
                const unsigned long long db = sdesc_mn(sa + ks * 2048, gbox, 1024, false);
                for (int j = 0; j < my_mt; ++j) {
                    // rows3: the four 32-row atoms of the M tile are the box seen from pixel rows
                    // 0, 1, 2, 3 (taps dx = -1, 0, 1 and an unused fourth): atoms 64 bytes apart
                    const unsigned long long da =
                        q.rows3 ? sdesc_mn(sa + g_bytes + j * xbox + ks * 2 * xsbo, 64, xsbo, true)
                                : sdesc_mn(sa + g_bytes + (unsigned)(j * q.spt) * xbox + ks * 2 * xsbo, xbox, xsbo,
                                           sw64);
                    umma(tmem + (unsigned)(j * q.N), da, db, id, (k > 0 || ks > 0) ? 1u : 0u);
                }
            }
            umma_commit(empty(st));
        }
        if (ok) umma_commit(done);
    }
    // Epilogue: warp w reads TMEM lanes 32w..32w+31 = rows of each M tile.
    const int cin = q.c0 + q.c1;
    float *part = q.partial + (size_t)chunk * 9 * cin * q.Cout;
    bool have = my_tiles > 0;
    if (have) {
        have = __all_sync(0xffffffffu, mbar_wait(done, 0));
        if (!have) ok = false;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    }
    const int row = 32 * warp + lane;
    for (int j = 0; j < my_mt; ++j) {
        int slot = slot0 + j * q.spt + row / q.aw, tap = slot / q.apt, atom = slot % q.apt;
        const int c = row % q.aw;
        if (q.rows3) {  // M tile (kernel row, atom); rows 32 s + c: tap dx = s - 1, s < 3
            const int i = mt0 + j, sx = row / 32;
            atom = i % q.apt;
            tap = 3 * (i / q.apt) + sx;
            slot = sx < 3 ? tap * q.apt + atom : 9 * q.apt;
        }
        int ci = -1;
        if (slot < 9 * q.apt) {
            if (atom < q.seg0) {
                if (q.aw * atom + c < q.c0) ci = q.aw * atom + c;
            } else if (q.aw * (atom - q.seg0) + c < q.c1) {
                ci = q.c0 + q.aw * (atom - q.seg0) + c;
            }
        }
        float *dst = part + ((size_t)tap * cin + ci) * q.Cout;
        for (int cb = 0; cb < q.N; cb += 16) {
            unsigned v[16];
            if (have) {
                tmem_ld16(tmem + ((unsigned)(32 * warp) << 16) + (unsigned)(j * q.N + cb), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            }
            if (ci < 0) continue;
            if (cb + 16 <= q.Cout) {
                float4 *d4 = reinterpret_cast<float4 *>(dst + cb);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    d4[e] = have ? make_float4(__uint_as_float(v[4 * e]), __uint_as_float(v[4 * e + 1]),
                                               __uint_as_float(v[4 * e + 2]), __uint_as_float(v[4 * e + 3]))
                                 : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            } else {
#pragma unroll
                for (int e = 0; e < 16; ++e)
                    if (cb + e < q.Cout) dst[cb + e] = have ? __uint_as_float(v[e]) : 0.0f;
            }
        }
    }
    if (!ok && lane == 0) atomicOr(&g_umma_status, 1u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(q.cols));
}

// Split of the weight gradient: atoms, slots per M tile, M tiles per CTA (TMEM and shared
// memory), 64-pixel tiles, tile ranges per CTA.
WgradTiles wgrad_tiles(int B, int H, int W, int c0, int c1, int Cout) {
    WgradTiles q{};
    q.B = B;
    q.H = H;
    q.W = W;
    q.Wb = 1;
    while (q.Wb < W && q.Wb < WG_KC) q.Wb *= 2;
    q.Hb = WG_KC / q.Wb;
    q.tx = (W + q.Wb - 1) / q.Wb;
    q.ty = (H + q.Hb - 1) / q.Hb;
    q.tiles = B * q.tx * q.ty;
    q.Cout = Cout;
    q.N = (Cout + 15) / 16 * 16;
    q.ga = (Cout + 63) / 64;
    q.c0 = c0;
    q.c1 = c1;
    // Atom width: the one that needs fewer M tiles (32-channel atoms waste less on inputs
    // like 48 + 32 channels); 64 on a tie (half the boxes).
    auto mtiles_for = [&](int aw) {
        const int apt = (c0 + aw - 1) / aw + (c1 + aw - 1) / aw;
        return (9 * apt + TM / aw - 1) / (TM / aw);
    };
    q.aw = mtiles_for(32) < mtiles_for(64) ? 32 : 64;
    q.seg0 = (c0 + q.aw - 1) / q.aw;
    q.apt = q.seg0 + (c1 + q.aw - 1) / q.aw;
    q.spt = TM / q.aw;
    q.mtiles = mtiles_for(q.aw);
    q.rows3 = q.aw == 32 && q.Wb == WG_KC && 3 * q.apt <= q.mtiles + q.apt;
    if (q.rows3) q.mtiles = 3 * q.apt;
    const unsigned gbytes = (unsigned)q.ga * WG_KC * 128,
                   mbytes = q.rows3 ? WG_ROWS3_STRIDE : (unsigned)q.spt * WG_KC * 2 * q.aw;  // 16 KB
    // M tiles per CTA: accumulators within 512 TMEM columns, and stages small enough for two
    // CTAs per SM (at most 4 rows3 boxes or 2 M tiles of 16 KB next to the G boxes); the M
    // tiles are then spread evenly over the CTA groups.
    const int cap = std::max(1, std::min({512 / q.N, q.rows3 ? 4 : 2, (int)((72 * 1024 - gbytes) / mbytes)}));
    const int groups = (q.mtiles + cap - 1) / cap;
    q.mt_per_cta = (q.mtiles + groups - 1) / groups;
    q.cols = 32;
    while (q.cols < q.mt_per_cta * q.N) q.cols *= 2;
    // About two CTAs per SM in total, but at least 4 tiles (256 pixels) per CTA: every CTA
    // writes its partial sums, which must stay small against its MMA work.
    const int target = 2 * 152;
    const int chunks = std::max(1, std::min((q.tiles + 3) / 4, (target + groups - 1) / groups));
    q.tiles_per_chunk = (q.tiles + chunks - 1) / chunks;
    // Stages: up to ~100 KB of them, so that two CTAs share an SM where the accumulators
    // allow (their MMA issue, not the tensor pipe, bounds these narrow GEMMs); at least two.
    const unsigned stage = gbytes + (unsigned)q.mt_per_cta * mbytes;
    q.stages = (int)std::max<size_t>(2, std::min<size_t>(WG_MAX_STAGES, (100 * 1024) / stage));
    return q;
}

// ---- host: tensor maps ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encoder(EncodeTiled *out) {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess ||
            qr != cudaDriverEntryPointSuccess || !p) {
            cudaGetLastError();
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return RT_ERR_CUDA;
        }
        fn = reinterpret_cast<EncodeTiled>(p);
    }
    *out = fn;
    return RT_OK;
}

// NHWC BF16 activations (B, H, W, C) read as boxes of 64 channels x bw x bh pixels (128-byte
// swizzle), or of 32 channels (64-byte swizzle) when narrow.
int map_activations(CUtensorMap *m, const bf16 *ptr, int B, int H, int W, int C, int bw, int bh, bool narrow) {
    EncodeTiled enc;
    int r = encoder(&enc);
    if (r != RT_OK) return r;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)(narrow ? KB / 2 : KB), (cuuint32_t)bw, (cuuint32_t)bh, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult e = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, narrow ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) {
        set_error("activation tensor map rejected (error " + std::to_string((int)e) + ")");
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

// Packed weights [rows][Kp] read as boxes of 64 K x N rows.
int map_weights(CUtensorMap *m, const bf16 *ptr, int Kp, int rows, int N) {
    EncodeTiled enc;
    int r = encoder(&enc);
    if (r != RT_OK) return r;
    const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
    const cuuint32_t box[2] = {(cuuint32_t)KB, (cuuint32_t)N};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult e = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) {
        set_error("weight tensor map rejected (error " + std::to_string((int)e) + ")");
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

// A layer's output (B, H, W, C), BF16 or FP32, written as boxes of FOLD_OUT pixels x all C
// channels from a plain [pixel][channel] shared-memory buffer.
int map_output(CUtensorMap *m, const void *ptr, int B, int H, int W, int C, bool f32) {
    EncodeTiled enc;
    int r = encoder(&enc);
    if (r != RT_OK) return r;
    const cuuint64_t es = f32 ? 4 : 2;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * es, (cuuint64_t)W * C * es, (cuuint64_t)H * W * C * es};
    const cuuint32_t box[4] = {(cuuint32_t)C, (cuuint32_t)FOLD_OUT, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult e = enc(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                           const_cast<void *>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) {
        set_error("output tensor map rejected (error " + std::to_string((int)e) + ")");
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

inline unsigned blocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

size_t packed_k(int c0, int c1) { return (size_t)9 * ((c0 + 63) / 64 + (c1 + 63) / 64) * 64; }

int conv_forward_umma(const ConvIn &in, int B, int H, int W, const bf16 *wpk, const float *bias, int Cout, bool relu,
                      bf16 *out_bf, float *out_f, bf16 *ups, cudaStream_t st, const FOut &fo, bool pdl) {
    if (fo.finish_out && (Cout % 16 != 0 || !fo.feat || fo.H > H || fo.W > W || out_f || out_bf)) {
        set_error("a finished convolution output needs Cout a multiple of 16, the features and no other output");
        return RT_ERR_ARG;
    }
    const bf16 *src0 = in.p0;
    if (in.up0) {
        if (!ups) {
            set_error("an upsampled convolution input needs scratch space");
            return RT_ERR_ARG;
        }
        const size_t n8 = (size_t)B * (H / 2) * (W / 2) * (in.c0 / 8);
        RT_CUDA_TRY(launch_pdl(k_upsample2, dim3(blocks(n8)), dim3(256), 0, st, pdl, in.p0, B, H / 2, W / 2, in.c0,
                               ups));
        src0 = ups;
    }
    ConvTiles q;
    q.H = H;
    q.W = W;
    q.Wb = 1;
    while (q.Wb < W && q.Wb < TM) q.Wb *= 2;
    q.Hb = TM / q.Wb;
    q.tx = (W + q.Wb - 1) / q.Wb;
    q.ty = (H + q.Hb - 1) / q.Hb;
    q.seg0 = (in.c0 + 63) / 64;
    q.cpt = q.seg0 + (in.c1 + 63) / 64;
    q.c0 = in.c0;
    q.c1 = in.c1;
    q.Cout = Cout;
    // N: the whole output in one tile when it fits the instruction (<= 256), else 128-wide tiles.
    q.N = Cout <= 256 ? (Cout + 15) / 16 * 16 : 128;
    q.nhalf = 32;  // TMEM columns of one accumulator
    while (q.nhalf < q.N) q.nhalf *= 2;
    q.groups = std::min(EPI_GROUPS, 512 / q.nhalf);
    q.mtiles = B * q.tx * q.ty;
    q.ntiles = q.mtiles * ((Cout + q.N - 1) / q.N);
    q.bias = bias;
    q.relu = relu ? 1 : 0;
    q.out_bf = out_bf;
    q.out_f = out_f;
    q.fin_feat = fo.feat;
    q.fin_out = fo.finish_out;
    q.fin_H = fo.H;
    q.fin_W = fo.W;
    q.tstore = 0;
    q.obuf = 0;
    q.wres = 0;
    q.narrow0 = q.narrow1 = 0;
    q.astage = 0;
    const bool rows = q.Wb == TM;  // every tile is 128 pixels of one row
    bool fold = false;
    size_t smem;
    if (rows) {
        const size_t kblk = (size_t)q.N * 128, wbytes = (size_t)9 * q.cpt * kblk;
        const size_t budget = 220 * 1024 - kFixed;
        q.narrow0 = DN_C32 && in.c0 <= 32;
        q.narrow1 = DN_C32 && in.c1 > 0 && in.c1 <= 32;
        const bool narrow_all = q.narrow0 && (in.c1 == 0 || q.narrow1);
        // folded tiles: the three horizontal taps in N (3 N <= 256) with resident weights
        const size_t fstage = 3 * (size_t)(narrow_all ? ROW32_BOX : ROW_BOX);
        fold = DN_FOLD && q.ntiles == q.mtiles && 3 * q.N <= 256 && wbytes + 2 * fstage <= budget;
        if (fold) {
            q.tx = (W + FOLD_OUT - 1) / FOLD_OUT;
            q.mtiles = q.ntiles = B * q.tx * q.ty;
            while (q.nhalf < 3 * q.N) q.nhalf *= 2;
            q.groups = std::min(EPI_GROUPS, 512 / q.nhalf);
            q.wres = 1;
            q.astage = (unsigned)fstage;
            // BF16 outputs leave through the groups' shared-memory buffers and TMA stores when
            // the buffers fit beside two stages.
            const int esz = out_f ? 4 : 2;
            const size_t obuf = ((size_t)FOLD_OUT * Cout * esz + 127) / 128 * 128;
            const size_t stores = (size_t)q.groups * obuf + 128;
            const bool one_out = (out_bf != nullptr) != (out_f != nullptr);
            q.tstore = (DN_TMA_STORE && one_out && !fo.finish_out && Cout % 8 == 0 &&
                        wbytes + stores + 2 * fstage <= budget)
                           ? (out_f ? 2 : 1)
                           : 0;
            q.obuf = q.tstore ? (unsigned)obuf : 0u;
            const size_t left = budget - wbytes - (q.tstore ? stores : 0);
            q.stages = (int)std::min<size_t>(MAX_STAGES, left / fstage);
            smem = kFixed + wbytes + q.stages * fstage + (q.tstore ? stores : 0);
        } else {
            q.astage = narrow_all ? HALO32_STAGE : HALO_STAGE;
            q.wres = q.ntiles == q.mtiles && wbytes + 4 * (size_t)q.astage <= budget;
            const size_t stage_bytes = q.astage + (q.wres ? 0 : 3 * kblk);
            const size_t avail = budget - (q.wres ? wbytes : 0);
            q.stages = (int)std::min<size_t>(MAX_STAGES, avail / stage_bytes);
            smem = kFixed + (q.wres ? wbytes : 0) + q.stages * stage_bytes;
        }
    } else {
        const size_t stage_bytes = (size_t)TM * 128 + (size_t)q.N * 128;
        q.stages = (int)std::min<size_t>(MAX_STAGES, (220 * 1024 - kFixed) / stage_bytes);
        smem = q.stages * stage_bytes + kFixed;
    }

    CUtensorMap tm0, tm1, tmw;
    const int bw = fold ? TM / EPI_WARPS : rows ? HALO : q.Wb, bh = rows ? 1 : q.Hb;
    int r = map_activations(&tm0, src0, B, H, W, in.c0, bw, bh, q.narrow0);
    if (r == RT_OK) {
        if (in.c1)
            r = map_activations(&tm1, in.p1, B, H, W, in.c1, bw, bh, q.narrow1);
        else
            tm1 = tm0;
    }
    if (r == RT_OK) r = map_weights(&tmw, wpk, (int)packed_k(in.c0, in.c1), Cout, q.N);
    CUtensorMap tmo = tmw;  // unused unless q.tstore
    if (r == RT_OK && q.tstore)
        r = map_output(&tmo, q.tstore == 2 ? static_cast<const void *>(out_f) : static_cast<const void *>(out_bf), B, H,
                       W, Cout, q.tstore == 2);
    if (r != RT_OK) return r;

    static bool configured = false;
    static int sms = 0;
    if (!configured) {
        for (const void *k : {(const void *)k_conv_umma<false>, (const void *)k_conv_rows<false>,
                              (const void *)k_conv_fold<false>, (const void *)k_conv_umma<true>,
                              (const void *)k_conv_rows<true>, (const void *)k_conv_fold<true>})
            RT_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448));
        int dev = 0;
        RT_CUDA_TRY(cudaGetDevice(&dev));
        RT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        configured = true;
    }
    const int grid = std::min(q.ntiles, sms);  // one persistent CTA per SM
    // The finished output layer is a separate instantiation, so that the other layers'
    // epilogues keep their registers.
    const bool xo = fo.finish_out != nullptr;
    // With pdl, launched with programmatic stream serialisation: the kernel may start while
    // the previous kernel on the stream drains; it waits for it (griddep_wait) before reading
    // activations. (Without the attribute griddep_wait returns at once.)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (DN_PDL && pdl) ? 1 : 0;
    if (fold)
        RT_CUDA_TRY(cudaLaunchKernelEx(&cfg, xo ? k_conv_fold<true> : k_conv_fold<false>, tm0, tm1, tmw, tmo, q));
    else if (rows)
        RT_CUDA_TRY(cudaLaunchKernelEx(&cfg, xo ? k_conv_rows<true> : k_conv_rows<false>, tm0, tm1, tmw, q));
    else
        RT_CUDA_TRY(cudaLaunchKernelEx(&cfg, xo ? k_conv_umma<true> : k_conv_umma<false>, tm0, tm1, tmw, q));
    return RT_OK;
}

int pack_weights(const float *w, int c0, int c1, int Cout, bf16 *wpk, bf16 *wpkd, cudaStream_t st) {
    if (wpk) {
        const size_t n = (size_t)Cout * packed_k(c0, c1);
        k_pack_fwd<float><<<blocks(n), 256, 0, st>>>(w, c0, c1, Cout, wpk, n);
    }
    if (wpkd) {
        const size_t n = (size_t)(c0 + c1) * packed_k(Cout, 0);
        k_pack_bwd<<<blocks(n), 256, 0, st>>>(w, c0 + c1, Cout, wpkd, n);
    }
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pack_weights_bf16(const bf16 *w, int c0, int c1, int Cout, bf16 *wpk, cudaStream_t st) {
    const size_t n = (size_t)Cout * packed_k(c0, c1);
    k_pack_fwd<bf16><<<blocks(n), 256, 0, st>>>(w, c0, c1, Cout, wpk, n);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pack_all(const float *params, const PackTable &tab, bf16 *wk, bf16 *wkd, cudaStream_t st) {
    k_pack_all<<<blocks(tab.fwd_total + tab.bwd_total), 256, 0, st>>>(params, tab, wk, wkd);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

// Scratch floats of conv_wgrad's partial sums: at most 2 x 152 tile ranges (wgrad_tiles).
size_t wgrad_partial_floats(long P, int Cin, int Cout) {
    (void)P;
    return (size_t)2 * 152 * 9 * Cin * Cout;
}

int conv_wgrad(const ConvIn &in, int B, int H, int W, const bf16 *g, int Cout, float *partial, float *dw, bf16 *ups,
               cudaStream_t st) {
    const bf16 *src0 = in.p0;
    if (in.up0) {
        if (!ups) {
            set_error("an upsampled convolution input needs scratch space");
            return RT_ERR_ARG;
        }
        const size_t n8 = (size_t)B * (H / 2) * (W / 2) * (in.c0 / 8);
        k_upsample2<<<blocks(n8), 256, 0, st>>>(in.p0, B, H / 2, W / 2, in.c0, ups);
        RT_CUDA_TRY(cudaGetLastError());
        src0 = ups;
    }
    if (Cout > 256) {
        set_error("the weight gradient takes at most 256 output channels");
        return RT_ERR_ARG;
    }
    WgradTiles q = wgrad_tiles(B, H, W, in.c0, in.c1, Cout);
    q.partial = partial;
    CUtensorMap tmg, tm0, tm1;
    const bool narrow = q.aw == 32;
    const int xbw = q.rows3 ? WG_KC + 4 : q.Wb;  // rows3: 68-pixel boxes from x0 - 1
    int r = map_activations(&tmg, g, B, H, W, Cout, q.Wb, q.Hb, false);
    if (r == RT_OK) r = map_activations(&tm0, src0, B, H, W, in.c0, xbw, q.Hb, narrow);
    if (r == RT_OK) {
        if (in.c1)
            r = map_activations(&tm1, in.p1, B, H, W, in.c1, xbw, q.Hb, narrow);
        else
            tm1 = tm0;
    }
    if (r != RT_OK) return r;
    static bool configured = false;
    if (!configured) {
        RT_CUDA_TRY(cudaFuncSetAttribute(k_wgrad_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448));
        configured = true;
    }
    const size_t stage = (size_t)q.ga * WG_KC * 128 +
                         (size_t)q.mt_per_cta * (q.rows3 ? WG_ROWS3_STRIDE : (size_t)q.spt * WG_KC * 2 * q.aw);
    const size_t smem = 1024 + q.stages * stage + 8 * (2 * WG_MAX_STAGES + 2);
    const int chunks = (q.tiles + q.tiles_per_chunk - 1) / q.tiles_per_chunk;
    const dim3 grid((unsigned)chunks, (unsigned)((q.mtiles + q.mt_per_cta - 1) / q.mt_per_cta), 1);
    k_wgrad_umma<<<grid, 128, smem, st>>>(tmg, tm0, tm1, q);
    RT_CUDA_TRY(cudaGetLastError());
    return reduce_chunks(partial, chunks, (size_t)9 * (in.c0 + in.c1) * Cout, dw, st);
}

int umma_status(bool clear) {
    unsigned s = 0;
    RT_CUDA_TRY(cudaMemcpyFromSymbol(&s, g_umma_status, sizeof(unsigned)));
    if (s && clear) {
        const unsigned z = 0;
        RT_CUDA_TRY(cudaMemcpyToSymbol(g_umma_status, &z, sizeof(unsigned)));
    }
    if (s) {
        set_error("a tensor-core convolution timed out waiting for its pipeline");
        return RT_ERR_TIMEOUT;
    }
    return RT_OK;
}

}  // namespace dn
}  // namespace rgb
