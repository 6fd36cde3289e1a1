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

// One panel step in two calls: pack the U panel (hi/lo TF32 B'' tiles),
// then update the column tiles [ct_lo, ct_hi) of the trailing block (the
// look-ahead schedule splits the update in two column ranges).
int tc_pack_b(const TcFront *fr, c64 *pool, int f_begin, int nfl, int k0, int max_trail, uint8_t *scratch,
              cudaStream_t st);
int tc_schur_cols(const TcFront *fr, c64 *pool, int f_begin, int nfl, int k0, int max_trail, int ct_lo,
                  int ct_hi, const uint8_t *scratch, int *err, cudaStream_t st);
int tc_prepare();

}  // namespace fdfd
