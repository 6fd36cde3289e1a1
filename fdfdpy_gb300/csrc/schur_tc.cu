// Tensor-core (tcgen05) Schur-complement update for the complex64 factor.
//
//   C[t0:m, t0:m] -= L[t0:m, k0:k0+w] * U[k0:k0+w, t0:m]      (complex64)
//
// The complex product is carried as one real GEMM:
//   A' (M x 2K): A'[i, 2l] = Re L[i,l],  A'[i, 2l+1] = Im L[i,l]
//   B'' (2K x 2N): B''[2l, 2j] = Re U,  B''[2l+1, 2j] = -Im U,
//                  B''[2l, 2j+1] = Im U, B''[2l+1, 2j+1] = Re U
//   (A' B'')[i, 2j] = Re C update, [i, 2j+1] = Im C update,
// so the accumulator's row i holds the (re, im) pairs of complex row i --
// exactly the interleaved column-major storage of the front.
//
// Precision: FP32-level products from TF32 tensor cores by the 3xTF32
// split (x = hi + lo, both TF32; A B ~ Ahi Bhi + Ahi Blo + Alo Bhi), the
// three MMAs accumulating in FP32 in tensor memory.
//
// Data movement: the GEMM CTA's four epilogue warps first write the A'
// rows of their 128-row tile (hi and lo, straight from the front) into
// tensor memory, one TMEM lane per row, so the MMAs read A from TMEM; a
// pack kernel writes each 32-column B'' tile (hi and lo) contiguously in
// global scratch in the canonical no-swizzle K-major core-matrix layout
// (8 rows x 16 bytes per core matrix), and a producer thread streams them
// into shared memory with bulk copies (cp.async.bulk, completion on an
// mbarrier per stage); one thread issues the 48 tcgen05.mma of a tile
// (16 K-steps x 3), tcgen05.commit signals the epilogue and releases the
// stage, and the four warps read the 128 x 64 FP32 accumulator back with
// tcgen05.ld (each warp its 32 TMEM lanes) and apply C -= acc with
// coalesced column-major stores.  All waits are bounded: on time-out the
// CTA records an error code, waits (bounded) for its own operations, frees
// its tensor memory and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "cplx.cuh"
#include "fdfd_internal.h"
#include "schur_tc.h"

namespace fdfd {
namespace tc {

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; returns false on time-out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// A from tensor memory (a_tmem: lane = row, one TF32 element per column),
// B from shared memory.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// 32 consecutive 32-bit columns of this thread's TMEM lane (warp w may
// address lanes 32 (w % 4) .. + 31).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]),
        "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]),
        "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// core matrices of 8 rows x 16 bytes; lbo = byte distance between the two
// core matrices of one K-step (K direction), sbo = between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, swizzle none
}
// Instruction descriptor: D f32, A/B tf32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- the GEMM ------------------------------------------------------------------
// One CTA = one 128-row tile of C and a run of up to kColTilesPerCta 32-column
// tiles (the launcher shortens the run when a launch would otherwise leave
// SMs idle: the last panels of the large fronts near the root),
// warp-specialized:
//   warps 0-7 (two per TMEM lane quarter, each with half of the columns)
//     first write the tile's A' rows (hi and lo TF32 parts of the L panel,
//     read straight from the front) into tensor memory -- thread = TMEM
//     lane = row -- so the MMAs read A from TMEM and only B from shared
//     memory; then they drain the accumulators (tcgen05.ld, C -= acc), the
//     next tile's C entries already loading (eight warps keep twice the C
//     loads in flight of four);
//   warp 9 (lane 0) streams the B'' tiles (hi, lo) through kStages shared-
//     memory stages, refilling a stage once the MMAs that read it are done;
//   warp 8 (lane 0) issues the 48 MMAs of each column tile (16 K-steps x 3)
//     into one of two TMEM accumulators and commits them to the epilogue's
//     barrier and to the stage's release barrier.
// TMEM columns: A hi [0,128), A lo [128,256), accumulators [256,384).
// Every wait is bounded; on time-out a thread records an error, the
// producer waits (bounded) for the copies it issued, and the CTA frees its
// tensor memory and returns.
constexpr int kColTilesPerCta = 16;  // longest column run of a CTA
constexpr int kMinColTiles = 2;      // shortest (the A' rows are loaded once per run)
constexpr int kStages = 3;
constexpr uint32_t kStageBytes = 2 * kBTileBytes;
constexpr uint32_t kSmemBytes = kStages * kStageBytes + 256;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kEpiWarps = 8;       // two per TMEM lane quarter, each half of a tile's columns
constexpr int kMmaWarp = kEpiWarps, kLoadWarp = kEpiWarps + 1;
constexpr int kCtaThreads = 32 * (kEpiWarps + 2);
constexpr uint32_t kTmemAlloc = 512;
constexpr uint32_t kTmemAHi = 0, kTmemALo = 2 * kPanel, kTmemAcc = 4 * kPanel;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// At most 128 registers a thread (one CTA: 40,960) so that a 256-thread,
// 80-register diagonal-block LU of the look-ahead stream (20,480) fits on
// the same SM beside it; shared memory fits likewise (196.9 + 33.3 KB).
__global__ void __maxnreg__(128)
    k_schur_tc(const TcFront *__restrict__ fr, c64 *pool, int f_begin, int k0, int ct_lo, int ct_hi,
               const uint8_t *scratch, int *err, int cpc) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const TcFront f = fr[f_begin + blockIdx.x];
    const int w = min(kPanel, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w, mt = f.m - t0;
    const int rt = blockIdx.y;
    const int cts = min((mt + kTileNc - 1) / kTileNc, ct_hi);
    const int ct0 = ct_lo + blockIdx.z * cpc;
    if (rt * kTileM >= mt || ct0 >= cts) return;
    const int J = min(cpc, cts - ct0);

    uint8_t *b_base = smem;
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *bar_a = &bars[0], *bar_full = &bars[1], *bar_free = &bars[1 + kStages];
    uint64_t *bar_mma = &bars[1 + 2 * kStages], *bar_epi = &bars[3 + 2 * kStages];
    uint32_t *tmem_slot = (uint32_t *)(bars + 5 + 2 * kStages);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        mbar_init(bar_a, kEpiWarps);
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&bar_full[s], 1);
            mbar_init(&bar_free[s], 1);
        }
        mbar_init(&bar_mma[0], 1);
        mbar_init(&bar_mma[1], 1);
        mbar_init(&bar_epi[0], kEpiWarps);
        mbar_init(&bar_epi[1], kEpiWarps);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kMmaWarp) {
        tmem_alloc(tmem_slot, kTmemAlloc);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == kLoadWarp) {
        if (lane == 0) {
            bool ok = true;
            int issued = 0;
            for (int j = 0; j < J; ++j) {
                const int s = j % kStages;
                if (j >= kStages && !mbar_wait_bounded(&bar_free[s], ((j / kStages) - 1) & 1, kWaitLimit)) {
                    ok = false;
                    break;
                }
                const uint8_t *gb = scratch + f.b_off + (size_t)(ct0 + j) * 2 * kBTileBytes;
                uint8_t *sb = b_base + s * kStageBytes;
                mbar_arrive_expect_tx(&bar_full[s], kStageBytes);
                bulk_g2s(sb, gb, kBTileBytes, &bar_full[s]);
                bulk_g2s(sb + kBTileBytes, gb + kBTileBytes, kBTileBytes, &bar_full[s]);
                issued = j + 1;
            }
            // the copies this thread issued complete before the CTA exits
            for (int j = (issued > kStages ? issued - kStages : 0); j < issued; ++j)
                mbar_wait_bounded(&bar_full[j % kStages], (j / kStages) & 1, kWaitLimit);
            if (!ok) atomicExch(err, 3);
        }
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            bool ok = mbar_wait_bounded(bar_a, 0, kWaitLimit);
            constexpr uint32_t idesc = idesc_tf32(kTileM, 2 * kTileNc);
            constexpr uint64_t b_step = (2 * (2 * kTileNc / 8) * 128) >> 4;
            const uint64_t bh00 = smem_desc(smem_u32(b_base), (2 * kTileNc / 8) * 128, 128);
            tc_fence_after();
            for (int j = 0; j < J && ok; ++j) {
                const int s = j % kStages, sidx = j & 1;
                if (!mbar_wait_bounded(&bar_full[s], (j / kStages) & 1, kWaitLimit)) { ok = false; break; }
                if (j >= 2 && !mbar_wait_bounded(&bar_epi[sidx], ((j - 2) >> 1) & 1, kWaitLimit)) {
                    ok = false;  // accumulator still being drained
                    break;
                }
                tc_fence_after();
                const uint64_t bh0 = bh00 + (uint64_t)((s * kStageBytes) >> 4);
                const uint64_t bl0 = bh0 + (uint64_t)(kBTileBytes >> 4);
                const uint32_t d = tmem + kTmemAcc + (uint32_t)(sidx * kTmemCols);
#pragma unroll
                for (int s2 = 0; s2 < 2 * kPanel / 8; ++s2) {
                    const uint32_t ah = tmem + kTmemAHi + 8 * s2, al = tmem + kTmemALo + 8 * s2;
                    mma_tf32_ts(d, ah, bh0 + s2 * b_step, idesc, s2 > 0 ? 1u : 0u);
                    mma_tf32_ts(d, ah, bl0 + s2 * b_step, idesc, 1);
                    mma_tf32_ts(d, al, bh0 + s2 * b_step, idesc, 1);
                }
                mma_commit(&bar_mma[sidx]);
                mma_commit(&bar_free[s]);
            }
            if (!ok) atomicExch(err, 1);
        }
    } else {
        // epilogue warp w owns TMEM lanes (tile rows) 32 (w % 4) .. + 31 and
        // half h = w / 4 of the columns: A' columns [64 h, 64 h + 64), complex
        // tile columns [16 h, 16 h + 16)
        const int q4 = warp & 3, h = warp >> 2;
        constexpr int kHalf = kTileNc / 2;
        const int row = t0 + rt * kTileM + q4 * 32 + lane;
        const bool live = row < f.m;
        c64 *F = pool + f.f_off;
        const int64_t ld = f.ld;
        const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
        // A' row: (Re, Im) of L[row, k0 + l] at columns (2l, 2l + 1), hi and lo parts
#pragma unroll 1
        for (int c = 2 * h; c < 2 * h + 2; ++c) {
            uint32_t hi[32], lo[32];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int l = 16 * c + q;
                c64 v = czero<c64>();
                if (live && l < w) v = F[row + (int64_t)(k0 + l) * ld];
                const float hx = tc_to_tf32(v.x), hy = tc_to_tf32(v.y);
                hi[2 * q] = __float_as_uint(hx);
                hi[2 * q + 1] = __float_as_uint(hy);
                lo[2 * q] = __float_as_uint(tc_to_tf32(v.x - hx));
                lo[2 * q + 1] = __float_as_uint(tc_to_tf32(v.y - hy));
            }
            tmem_st32(lane_base + kTmemAHi + 32 * c, hi);
            tmem_st32(lane_base + kTmemALo + 32 * c, lo);
        }
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_a);

        c64 cv[kHalf], nv[kHalf];
#pragma unroll
        for (int q = 0; q < kHalf; ++q) {
            const int col = t0 + ct0 * kTileNc + kHalf * h + q;
            cv[q] = (live && col < f.m) ? F[row + (int64_t)col * ld] : czero<c64>();
            nv[q] = czero<c64>();
        }
        for (int j = 0; j < J; ++j) {
            const int sidx = j & 1;
            const int colbase = t0 + (ct0 + j) * kTileNc + kHalf * h;
            // the next tile's C entries load while this tile's MMAs finish,
            // and the one after that is prefetched into L2 (no registers)
            if (j + 1 < J) {
#pragma unroll
                for (int q = 0; q < kHalf; ++q) {
                    const int col = colbase + kTileNc + q;
                    nv[q] = (live && col < f.m) ? F[row + (int64_t)col * ld] : czero<c64>();
                }
            }
            if (j + 2 < J && live) {
#pragma unroll
                for (int q = 0; q < kHalf; ++q) {
                    const int col = colbase + 2 * kTileNc + q;
                    if (col < f.m)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(F + row + (int64_t)col * ld) : "memory");
                }
            }
            const bool got = mbar_wait_bounded(&bar_mma[sidx], (j >> 1) & 1, kWaitLimit);
            if (!__all_sync(0xffffffffu, got)) {
                if (lane == 0) atomicExch(err, 2);
                break;
            }
            tc_fence_after();
            const uint32_t base = lane_base + kTmemAcc + (uint32_t)(sidx * kTmemCols + 2 * kHalf * h);
#pragma unroll
            for (int c0 = 0; c0 < 2 * kHalf; c0 += 16) {
                uint32_t r[16];
                tmem_ld16(base + (uint32_t)c0, r);
                tmem_ld_wait();
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    cv[c0 / 2 + q].x -= __uint_as_float(r[2 * q]);
                    cv[c0 / 2 + q].y -= __uint_as_float(r[2 * q + 1]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_epi[sidx]);
            if (live) {
#pragma unroll
                for (int q = 0; q < kHalf; ++q) {
                    const int col = colbase + q;
                    if (col < f.m) F[row + (int64_t)col * ld] = cv[q];
                }
            }
#pragma unroll
            for (int q = 0; q < kHalf; ++q) cv[q] = nv[q];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarp) tmem_dealloc(tmem, kTmemAlloc);
}

}  // namespace tc

// ---- host launchers ------------------------------------------------------------
int tc_schur_cols(const TcFront *fr, c64 *pool, int f_begin, int nfl, int k0, int max_trail, int ct_lo,
                  int ct_hi, const uint8_t *scratch, int *err, cudaStream_t st) {
    const int rts = (max_trail + kTileM - 1) / kTileM;
    const int cts = std::min((max_trail + kTileNc - 1) / kTileNc, ct_hi) - ct_lo;
    if (rts < 1 || cts < 1) return FDFD_OK;
    // column run per CTA: the longest that still gives about two CTAs per SM
    // (one CTA is resident per SM: TMEM and shared memory), at least two tiles
    static int sms = 0;
    if (!sms) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        sms = (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0) ? n : 152;
    }
    const int64_t tiles = (int64_t)nfl * rts * cts;
    const int cpc = (int)std::max<int64_t>(tc::kMinColTiles,
                                           std::min<int64_t>(tc::kColTilesPerCta, (tiles + 2 * sms - 1) / (2 * sms)));
    const int cgs = (cts + cpc - 1) / cpc;
    tc::k_schur_tc<<<dim3(nfl, rts, cgs), tc::kCtaThreads, tc::kSmemBytes, st>>>(fr, pool, f_begin, k0, ct_lo,
                                                                                ct_hi, scratch, err, cpc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string("schur_tc: ") + cudaGetErrorString(e));
    return FDFD_OK;
}

int tc_prepare() {
    cudaError_t e = cudaFuncSetAttribute(tc::k_schur_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::kSmemBytes);
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string("schur_tc attr: ") + cudaGetErrorString(e));
    return FDFD_OK;
}

}  // namespace fdfd
