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
// Data movement: a pack kernel writes each 128-row A' tile and each
// 64-column B'' tile (hi and lo) contiguously in global scratch in the
// canonical no-swizzle K-major core-matrix layout of tcgen05 (8 rows x 16
// bytes per core matrix); the GEMM CTA pulls them into shared memory with
// four bulk copies (cp.async.bulk, completion on an mbarrier), one thread
// issues the 48 tcgen05.mma of the tile (16 K-steps x 3), tcgen05.commit
// signals a second mbarrier, and four warps read the 128 x 64 FP32
// accumulator back with tcgen05.ld (each warp its 32 TMEM lanes) and apply
// C -= acc with coalesced column-major stores.  All waits are bounded:
// on time-out the CTA records an error code, waits (bounded) for its own
// operations, frees its tensor memory and returns.
#include <cuda_runtime.h>

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
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
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

// ---- packing ---------------------------------------------------------------
// Byte offset of real element (row r in [0,rows), k in [0,128)) inside a
// packed K-major tile with `groups` 8-row groups.
__device__ __forceinline__ uint32_t pack_off(int r, int k, int groups) {
    const int s = k >> 3, ki = (k >> 2) & 1, e = k & 3, mi = r >> 3, rr = r & 7;
    return (uint32_t)(s * (2 * groups * 128) + ki * (groups * 128) + mi * 128 + rr * 16 + e * 4);
}

// A' tiles of every front of a level: grid (front, row tile), 256 threads.
__global__ void k_pack_a(const TcFront *__restrict__ fr, const c64 *__restrict__ pool, int f_begin, int k0,
                         uint8_t *scratch) {
    const TcFront f = fr[f_begin + blockIdx.x];
    const int w = min(kPanel, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w, mt = f.m - t0;
    const int rt = blockIdx.y;
    if (rt * kTileM >= mt) return;
    uint8_t *hi = scratch + f.a_off + (size_t)rt * 2 * kATileBytes;
    uint8_t *lo = hi + kATileBytes;
    const c64 *F = pool + f.f_off;
    for (int idx = threadIdx.x; idx < kTileM * kPanel; idx += blockDim.x) {
        const int r = idx % kTileM, l = idx / kTileM;
        const int row = t0 + rt * kTileM + r;
        c64 v = czero<c64>();
        if (row < f.m && l < w) v = F[row + (int64_t)(k0 + l) * f.ld];
        const float h0 = to_tf32(v.x), h1 = to_tf32(v.y);
        const uint32_t o0 = pack_off(r, 2 * l, kTileM / 8), o1 = pack_off(r, 2 * l + 1, kTileM / 8);
        *(float *)(hi + o0) = h0;
        *(float *)(hi + o1) = h1;
        *(float *)(lo + o0) = to_tf32(v.x - h0);
        *(float *)(lo + o1) = to_tf32(v.y - h1);
    }
}

// B'' tiles: grid (front, column tile), 256 threads.
__global__ void k_pack_b(const TcFront *__restrict__ fr, const c64 *__restrict__ pool, int f_begin, int k0,
                         uint8_t *scratch) {
    const TcFront f = fr[f_begin + blockIdx.x];
    const int w = min(kPanel, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w, mt = f.m - t0;
    const int ct = blockIdx.y;
    if (ct * kTileNc >= mt) return;
    uint8_t *hi = scratch + f.b_off + (size_t)ct * 2 * kBTileBytes;
    uint8_t *lo = hi + kBTileBytes;
    const c64 *F = pool + f.f_off;
    constexpr int G = 2 * kTileNc / 8;
    for (int idx = threadIdx.x; idx < kTileNc * kPanel; idx += blockDim.x) {
        const int l = idx % kPanel, j = idx / kPanel;
        const int col = t0 + ct * kTileNc + j;
        c64 v = czero<c64>();
        if (col < f.m && l < w) v = F[(k0 + l) + (int64_t)col * f.ld];
        const float re_h = to_tf32(v.x), im_h = to_tf32(v.y);
        const float re_l = to_tf32(v.x - re_h), im_l = to_tf32(v.y - im_h);
        // (2l, 2j) = re, (2l+1, 2j) = -im, (2l, 2j+1) = im, (2l+1, 2j+1) = re;
        // B'' is stored N-row major over K: row n' = 2j + c, column k' = 2l + a.
        const int n0 = 2 * j, n1 = 2 * j + 1, ka = 2 * l, kb = 2 * l + 1;
        *(float *)(hi + pack_off(n0, ka, G)) = re_h;
        *(float *)(hi + pack_off(n0, kb, G)) = -im_h;
        *(float *)(hi + pack_off(n1, ka, G)) = im_h;
        *(float *)(hi + pack_off(n1, kb, G)) = re_h;
        *(float *)(lo + pack_off(n0, ka, G)) = re_l;
        *(float *)(lo + pack_off(n0, kb, G)) = -im_l;
        *(float *)(lo + pack_off(n1, ka, G)) = im_l;
        *(float *)(lo + pack_off(n1, kb, G)) = re_l;
    }
}

// ---- the GEMM ------------------------------------------------------------------
// One CTA = one 128-row tile of C and up to kColTilesPerCta 32-column tiles.
// Warp 4 (lane 0) is the control thread: it pulls the A tile (hi, lo) once,
// then for each column tile pulls B (hi, lo) into the single B buffer once
// the previous tile's MMAs have released it, and issues 48 MMAs into one of
// two TMEM accumulators.  Warps 0-3 drain the other accumulator meanwhile
// (tcgen05.ld of their 32 TMEM lanes, C -= acc) and hand it back through an
// mbarrier.  Every wait is bounded.
constexpr int kColTilesPerCta = 8;
constexpr uint32_t kSmemBytes = 2 * kATileBytes + 2 * kBTileBytes + 256;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kCtaThreads = 160;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(kCtaThreads, 1)
    k_schur_tc(const TcFront *__restrict__ fr, c64 *pool, int f_begin, int k0, const uint8_t *scratch,
               int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const TcFront f = fr[f_begin + blockIdx.x];
    const int w = min(kPanel, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w, mt = f.m - t0;
    const int rt = blockIdx.y;
    const int cts = (mt + kTileNc - 1) / kTileNc;
    const int ct0 = blockIdx.z * kColTilesPerCta;
    if (rt * kTileM >= mt || ct0 >= cts) return;
    const int J = min(kColTilesPerCta, cts - ct0);

    uint8_t *a_hi = smem, *a_lo = smem + kATileBytes;
    uint8_t *b_hi = smem + 2 * kATileBytes, *b_lo = b_hi + kBTileBytes;
    uint64_t *bars = (uint64_t *)(smem + 2 * kATileBytes + 2 * kBTileBytes);
    uint64_t *bar_a = &bars[0], *bar_b = &bars[1], *bar_mma = &bars[2], *bar_epi = &bars[4];
    uint32_t *tmem_slot = (uint32_t *)(bars + 6);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        mbar_init(bar_a, 1);
        mbar_init(bar_b, 1);
        mbar_init(&bar_mma[0], 1);
        mbar_init(&bar_mma[1], 1);
        mbar_init(&bar_epi[0], 4);
        mbar_init(&bar_epi[1], 4);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        tmem_alloc(tmem_slot, 2 * kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 4) {
        if (lane == 0) {
            bool ok = true;
            const uint8_t *ga = scratch + f.a_off + (size_t)rt * 2 * kATileBytes;
            mbar_arrive_expect_tx(bar_a, 2 * kATileBytes);
            bulk_g2s(a_hi, ga, kATileBytes, bar_a);
            bulk_g2s(a_lo, ga + kATileBytes, kATileBytes, bar_a);
            ok = mbar_wait_bounded(bar_a, 0, kWaitLimit);
            constexpr uint32_t idesc = idesc_tf32(kTileM, 2 * kTileNc);
            constexpr uint32_t a_step = 2 * (kTileM / 8) * 128;
            constexpr uint32_t b_step = 2 * (2 * kTileNc / 8) * 128;
            const uint32_t sa_hi = smem_u32(a_hi), sa_lo = smem_u32(a_lo);
            const uint32_t sb_hi = smem_u32(b_hi), sb_lo = smem_u32(b_lo);
            for (int j = 0; j < J && ok; ++j) {
                const int sidx = j & 1;
                if (j >= 1 && !mbar_wait_bounded(&bar_mma[(j - 1) & 1], ((j - 1) >> 1) & 1, kWaitLimit)) {
                    ok = false;  // B buffer still in use
                    break;
                }
                const uint8_t *gb = scratch + f.b_off + (size_t)(ct0 + j) * 2 * kBTileBytes;
                mbar_arrive_expect_tx(bar_b, 2 * kBTileBytes);
                bulk_g2s(b_hi, gb, kBTileBytes, bar_b);
                bulk_g2s(b_lo, gb + kBTileBytes, kBTileBytes, bar_b);
                if (!mbar_wait_bounded(bar_b, j & 1, kWaitLimit)) { ok = false; break; }
                if (j >= 2 && !mbar_wait_bounded(&bar_epi[sidx], ((j - 2) >> 1) & 1, kWaitLimit)) {
                    ok = false;  // accumulator still being drained
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(sidx * kTmemCols);
                for (int s2 = 0; s2 < 2 * kPanel / 8; ++s2) {
                    const uint64_t ah = smem_desc(sa_hi + s2 * a_step, (kTileM / 8) * 128, 128);
                    const uint64_t al = smem_desc(sa_lo + s2 * a_step, (kTileM / 8) * 128, 128);
                    const uint64_t bh = smem_desc(sb_hi + s2 * b_step, (2 * kTileNc / 8) * 128, 128);
                    const uint64_t bl = smem_desc(sb_lo + s2 * b_step, (2 * kTileNc / 8) * 128, 128);
                    mma_tf32(d, ah, bh, idesc, s2 > 0 ? 1u : 0u);
                    mma_tf32(d, ah, bl, idesc, 1);
                    mma_tf32(d, al, bh, idesc, 1);
                }
                mma_commit(&bar_mma[sidx]);
            }
            if (!ok) atomicExch(err, 1);
        }
    } else {
        // epilogue warps 0-3: warp w owns TMEM lanes (accumulator rows) 32w..32w+31
        const int row = t0 + rt * kTileM + warp * 32 + lane;
        c64 *F = pool + f.f_off;
        const int64_t ld = f.ld;
        for (int j = 0; j < J; ++j) {
            const int sidx = j & 1;
            const int colbase = t0 + (ct0 + j) * kTileNc;
            // prefetch this row's 32 C entries of the tile while the MMAs run
            c64 cv[kTileNc];
            const bool live = row < f.m;
#pragma unroll
            for (int q = 0; q < kTileNc; ++q) {
                const int col = colbase + q;
                cv[q] = (live && col < f.m) ? F[row + (int64_t)col * ld] : czero<c64>();
            }
            const bool got = mbar_wait_bounded(&bar_mma[sidx], (j >> 1) & 1, kWaitLimit);
            if (!__all_sync(0xffffffffu, got)) {
                if (lane == 0) atomicExch(err, 2);
                break;
            }
            tc_fence_after();
            const uint32_t base = tmem + (uint32_t)(sidx * kTmemCols) + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int c0 = 0; c0 < 2 * kTileNc; c0 += 16) {
                uint32_t r[16];
                tmem_ld16(base + (uint32_t)c0, r);
                tmem_ld_wait();
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    cv[c0 / 2 + q].x -= __uint_as_float(r[2 * q]);
                    cv[c0 / 2 + q].y -= __uint_as_float(r[2 * q + 1]);
                }
            }
            if (live) {
#pragma unroll
                for (int q = 0; q < kTileNc; ++q) {
                    const int col = colbase + q;
                    if (col < f.m) F[row + (int64_t)col * ld] = cv[q];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_epi[sidx]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) tmem_dealloc(tmem, 2 * kTmemCols);
}

}  // namespace tc

// ---- host launchers ------------------------------------------------------------
int tc_schur_step(const TcFront *fr, c64 *pool, int f_begin, int nfl, int k0, int max_trail,
                  uint8_t *scratch, int *err, cudaStream_t st) {
    const int rts = (max_trail + kTileM - 1) / kTileM;
    const int cts = (max_trail + kTileNc - 1) / kTileNc;
    if (rts < 1 || cts < 1) return FDFD_OK;
    tc::k_pack_a<<<dim3(nfl, rts), 256, 0, st>>>(fr, pool, f_begin, k0, scratch);
    tc::k_pack_b<<<dim3(nfl, cts), 256, 0, st>>>(fr, pool, f_begin, k0, scratch);
    const int cgs = (cts + tc::kColTilesPerCta - 1) / tc::kColTilesPerCta;
    tc::k_schur_tc<<<dim3(nfl, rts, cgs), tc::kCtaThreads, tc::kSmemBytes, st>>>(fr, pool, f_begin, k0, scratch,
                                                                                err);
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
