// Tensor-core Schur update of the complex64 factor (schur_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cplx.cuh"

namespace fdfd {

constexpr int kPanel = 64;    // panel width (the factor's NB)
constexpr int kTileM = 128;   // complex rows per tile (= MMA M, TMEM lanes)
constexpr int kTileNc = 32;   // complex columns per tile (MMA N = 64 reals)
constexpr uint32_t kBTileBytes = 2 * kTileNc * 2 * kPanel * 4;  // 32 KB
constexpr uint32_t kTmemCols = 2 * kTileNc;                     // FP32 accumulator columns

// TF32 rounding (round to nearest, ties away) of an FP32 value.
__device__ __forceinline__ float tc_to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Byte offset of real element (row r, k in [0, 128)) inside a packed
// K-major tile with `groups` 8-row groups (canonical no-swizzle layout of
// tcgen05: core matrices of 8 rows x 16 bytes; a K-step of 8 holds two core
// matrices along K, groups * 128 bytes apart; 8-row groups 128 bytes apart).
__device__ __forceinline__ uint32_t tc_pack_off(int r, int k, int groups) {
    const int s = k >> 3, ki = (k >> 2) & 1, e = k & 3, mi = r >> 3, rr = r & 7;
    return (uint32_t)(s * (2 * groups * 128) + ki * (groups * 128) + mi * 128 + rr * 16 + e * 4);
}

// Stores U[l][j] (panel row l, tile column j) into a B'' tile pair as the
// 2 x 2 real block [[re, im], [-im, re]] (rows 2l, 2l+1 of K; columns 2j,
// 2j+1 of N), hi and lo TF32 parts.
__device__ __forceinline__ void tc_store_b(uint8_t *hi, uint8_t *lo, int l, int j, c64 v) {
    constexpr int G = 2 * kTileNc / 8;
    const float re_h = tc_to_tf32(v.x), im_h = tc_to_tf32(v.y);
    const float re_l = tc_to_tf32(v.x - re_h), im_l = tc_to_tf32(v.y - im_h);
    const int n0 = 2 * j, n1 = 2 * j + 1, ka = 2 * l, kb = 2 * l + 1;
    *(float *)(hi + tc_pack_off(n0, ka, G)) = re_h;
    *(float *)(hi + tc_pack_off(n0, kb, G)) = -im_h;
    *(float *)(hi + tc_pack_off(n1, ka, G)) = im_h;
    *(float *)(hi + tc_pack_off(n1, kb, G)) = re_h;
    *(float *)(lo + tc_pack_off(n0, ka, G)) = re_l;
    *(float *)(lo + tc_pack_off(n0, kb, G)) = -im_l;
    *(float *)(lo + tc_pack_off(n1, ka, G)) = im_l;
    *(float *)(lo + tc_pack_off(n1, kb, G)) = re_l;
}

struct TcFront {
    int64_t f_off;         // front block offset in the pool (elements)
    int64_t a_off, b_off;  // packed-operand offsets in the scratch (bytes; a_off unused)
    int32_t m, p, ld, pad;
};

// Bytes of packed-operand scratch (the B'' tiles) for one front of size m, p.
inline int64_t tc_front_scratch(int m, int p, int64_t *a_bytes) {
    const int w = p < kPanel ? p : kPanel;
    const int64_t trail = (int64_t)m - w;
    const int64_t cts = (trail + kTileNc - 1) / kTileNc;
    *a_bytes = 0;
    return cts * 2 * (int64_t)kBTileBytes;
}

// Update of the column tiles [ct_lo, ct_hi) of a panel step's trailing
// block from the packed B'' tiles of the U panel (written by the panel's
// triangular update); the look-ahead schedule splits the columns in two.
int tc_schur_cols(const TcFront *fr, c64 *pool, int f_begin, int nfl, int k0, int max_trail, int ct_lo,
                  int ct_hi, const uint8_t *scratch, int *err, cudaStream_t st);
int tc_prepare();

}  // namespace fdfd
