// Multifrontal sparse LU of the FDFD operator on the GPU.
//
// Replaces the factor/solve of pardisoSolver(A, mtype=13) and of scipy's
// spsolve in solver_direct (fdfdpy/linalg.py:122-149).
//
// Storage: every front f of the nested-dissection tree owns a dense
// column-major ld_f x m_f block in one device pool.  After factorization
// the block holds
//   * below the diagonal blocks: L (unit lower, multipliers),
//   * right of the diagonal blocks: U,
//   * each nb x nb diagonal block: inv(L_kk) strictly below its diagonal
//     and inv(U_kk) on and above it (both triangular inverses are used by
//     the TRSM-as-GEMM updates and by the blocked triangular solves); the
//     whole fronts of the levels solved one warp per front keep these
//     inverses only inside 16 x 16 diagonal blocks (blocked format),
//   * the trailing (m-p) x (m-p) block: the update (Schur complement)
//     matrix that the parent gathers by its extend-add.
// The operator is factored scaled by sigma = 1/max|diag(A)| so that the
// complex64 factor stays well inside float range (Hz entries reach 1e21).
//
// Pivoting is static: no row exchanges, and a pivot below a threshold
// relative to the scaled operator (1e-5 for complex64, sqrt(eps) for
// complex128, or the caller's) is replaced and counted; the FP64
// iterative refinement absorbs the perturbation.
//
// Parallel schedule: fronts are processed level by level (leaves first).
// Each launch handles every front of a level: grid.x = front, grid.y/z =
// tiles of that front.  Fronts above the leaves are written whole by the
// parent-side extend-add (the pool is never cleared); the leaves assemble
// their fronts inside their LU launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <string>
#include <type_traits>
#include <vector>

#include "cplx.cuh"
#include "profile.h"
#include "schur_tc.h"
#include "stencil.cuh"

namespace fdfd {

int norms_device(const void *v, int64_t n, int ncol, double *partial, double *out_dev,
                 cudaStream_t st);
size_t norms_partial_count(int ncol);
int apply_device(const OpDev &o, const void *x, const void *b, void *out, int nrhs, int mode,
                 cudaStream_t st);

namespace {

constexpr int NB = 64;        // panel width
constexpr int BM = 64;        // GEMM tile rows
constexpr int BN = 64;        // GEMM tile cols
constexpr int BK = 16;        // GEMM K chunk
constexpr int kRowsPerCta = 256;
constexpr int kDotParts = 152 * 2;  // partial sums per GMRES dot product

struct FrontD {
    int64_t f_off;  // element offset of the dense block in the pool
    int32_t m, p, ld, voff;
    int32_t c0, c1;
};

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(FDFD_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// ---------------------------------------------------------------------------
// Operator coefficients [5][n] (centre, then the four neighbour directions)
// evaluated once per factorization.  stencil_row evaluates the coefficient
// formulas in FP64, whose rate on this GPU is a small fraction of FP32, so
// the assembly of the fronts and every refinement residual read the stored
// values instead of re-deriving them per cell (and per neighbour for A^T).
// coef[d * ld + k]: ld = n for one operator, the batch's total for problem
// b's slice of a batch (coef then points at the slice).
//
// The values are stencil_row's, bit for bit, with about half of its FP64
// operations:
// * a scaling by -1/dx (-1/dy) is the negation of the one by +1/dx (+1/dy)
//   (rounding to nearest is symmetric), so each product of two negated
//   factors is the product of the positive ones, the two centre products of
//   a direction that carry one minus sign are its negated neighbour
//   coefficients, and the centre is the diagonal term minus
//   (c_xm + c_xp) + (c_ym + c_yp), summed in stencil_row's order;
// * every 1/eps_x and 1/eps_y (Hz) serves two cells: a thread walks down its
//   column carrying 1/eps_x, eps_r and the 1/s_xb factor of the next row,
//   and a block hands 1/eps_y of each cell to the thread of the previous
//   column through shared memory.
// Block: kCoefCols consecutive columns j0 + t over the rows [r0, r1) of one
// run; grid: (column blocks, row runs), one wave of CTAs where the grid
// allows, so that every CTA has the same number of rows (+-1).
constexpr int kCoefCols = 256;
__global__ void __launch_bounds__(kCoefCols) k_coef(OpDev o, double2 *coef, int64_t ld, int rows_per_run) {
    __shared__ double s_ty[2][kCoefCols + 1];
    const int Nx = o.Nx, Ny = o.Ny, t = threadIdx.x;
    const int j0 = blockIdx.x * kCoefCols, j = j0 + t;
    const int r0 = blockIdx.y * rows_per_run, r1 = min(r0 + rows_per_run, Nx);
    if (r0 >= Nx) return;  // block-uniform
    const bool live = j < Ny;
    const int jc = live ? j : Ny - 1;  // idle threads of the last column block evaluate a valid cell
    const int jp = (jc == Ny - 1) ? 0 : jc + 1;
    const int jm = (jc == 0) ? Ny - 1 : jc - 1;
    // The one thread of the block whose next column (jp) is not the next
    // thread's: the last live column (next column 0) or the block's last
    // thread (next column j0 + kCoefCols); that column is jx.
    const int te = min(kCoefCols - 1, Ny - 1 - j0);
    const int jx = (j0 + kCoefCols < Ny) ? j0 + kCoefCols : 0;
    const bool hz = o.pol == FDFD_POL_HZ;
    const double vx = o.invdx, vy = o.invdy;
    double2 fy = c_scale_rn(o.isyf[jc], vy);
    if (!hz) fy = c_scale_rn(fy, o.invmu);  // (Dyf * 1 / MU_0_)
    const double2 by0 = c_scale_rn(o.isyb[jc], vy), by1 = c_scale_rn(o.isyb[jp], vy);
    double2 bx0 = c_scale_rn(o.isxb[r0], vx);
    double e0 = eps_e(o, r0, jc);
    double tx0 = hz ? inv_eps_x(o, r0, jc) : 0.0;
    int buf = 0;
    for (int i = r0; i < r1; ++i) {
        const int ip = (i == Nx - 1) ? 0 : i + 1;
        double2 fx = c_scale_rn(o.isxf[i], vx);
        if (!hz) fx = c_scale_rn(fx, o.invmu);
        const double2 bx1 = c_scale_rn(o.isxb[ip], vx);
        const double e1 = eps_e(o, ip, jc);
        double2 c1, c2, c3, c4, diag;
        if (hz) {
            // inv_eps_x(ip, j): the row below ip's is i; inv_eps_y(i, j)
            const double tx1 = __ddiv_rn(1.0, o.averaging ? __dmul_rn(__dadd_rn(e0, e1), 0.5) : e1);
            const double ty0 = __ddiv_rn(1.0, o.averaging ? __dmul_rn(__dadd_rn(eps_e(o, i, jm), e0), 0.5) : e0);
            s_ty[buf][t] = ty0;
            if (t == kCoefCols - 1) s_ty[buf][kCoefCols] = inv_eps_y(o, i, jx);
            __syncthreads();
            const double ty1 = s_ty[buf][t == te ? kCoefCols : t + 1];  // inv_eps_y(i, jp)
            buf ^= 1;  // the next row writes the other buffer; the one after passes this row's barrier first
            c1 = c_mul_rn(c_scale_rn(fx, tx0), bx0);
            c2 = c_mul_rn(c_scale_rn(fx, tx1), bx1);
            c3 = c_mul_rn(c_scale_rn(fy, ty0), by0);
            c4 = c_mul_rn(c_scale_rn(fy, ty1), by1);
            diag = make_double2(o.w2mu, 0.0);
            tx0 = tx1;
        } else {
            c1 = c_mul_rn(fx, bx0);
            c2 = c_mul_rn(fx, bx1);
            c3 = c_mul_rn(fy, by0);
            c4 = c_mul_rn(fy, by1);
            diag = make_double2(__dmul_rn(o.w2, e0), 0.0);
        }
        if (live) {
            const int64_t k = (int64_t)i * Ny + j;
            double2 ctr = c_sub_rn(diag, c_add_rn(c_add_rn(c1, c2), c_add_rn(c3, c4)));
            if (o.eps_add) ctr.x = __dadd_rn(ctr.x, __dmul_rn(o.w2e0L, o.eps_add[k]));
            if (o.diag_add) ctr = c_add_rn(ctr, o.diag_add[k]);
            coef[k] = ctr;
            coef[ld + k] = c1;
            coef[2 * ld + k] = c2;
            coef[3 * ld + k] = c3;
            coef[4 * ld + k] = c4;
        }
        bx0 = bx1;
        e0 = e1;
    }
}

// max |A[k,k]| over the grid, as the bit pattern of a non-negative double.
// hypot (many FP64 operations on this GPU) is evaluated once a thread, for
// the entry of largest squared modulus, and for the entries within 1e-12
// of that one's squared modulus that differ from it; an entry outside the
// margin has a smaller hypot than the kept one (the rounding of both is far
// below 1e-12), so the result is the maximum of hypot over every entry.
__global__ void k_maxdiag(OpDev o, unsigned long long *out) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    double mx = 0.0, s2max = -1.0;  // no entry kept yet
    double2 best = make_double2(0.0, 0.0);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        double2 c0;
        if (o.stencil) {
            c0 = o.stencil[k];  // stored coefficients: the centre row of [5][n]
        } else {
            double2 c[5];
            stencil_row(o, (int)(k / o.Ny), (int)(k % o.Ny), c);
            c0 = c[0];
        }
        const double s2 = c0.x * c0.x + c0.y * c0.y;
        if (s2 > s2max * (1.0 + 1e-12)) {
            best = c0;  // a clearly larger entry: the previous one cannot be the maximum
            s2max = s2;
        } else if (!(s2 < s2max * (1.0 - 1e-12)) && (c0.x != best.x || c0.y != best.y)) {
            mx = fmax(mx, hypot(c0.x, c0.y));  // within the margin (or NaN): evaluated
        }
    }
    if (s2max >= 0.0) mx = fmax(mx, hypot(best.x, best.y));
    for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

// Scatter the operator's entries into the fronts: row and column of each
// pivot variable, restricted to variables of the same front (the entries
// towards already-eliminated variables were assembled by descendants).
template <typename T>
__global__ void k_assemble_fronts(OpDev o, const FrontD *__restrict__ fr,
                                  const int32_t *__restrict__ var_front,
                                  const int32_t *__restrict__ var_loc,
                                  const int32_t *__restrict__ nbr_loc,
                                  const unsigned long long *maxdiag, T *pool, int f_lo, int f_hi) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    const double sigma = 1.0 / __longlong_as_double((long long)*maxdiag);
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x) {
        // only the variables of fronts [f_lo, f_hi)
        if (var_front[s] < f_lo || var_front[s] >= f_hi) continue;
        const int i = (int)(s / o.Ny), j = (int)(s % o.Ny);
        const FrontD f = fr[var_front[s]];
        T *F = pool + f.f_off;
        const int64_t ld = f.ld;
        const int k = var_loc[s];
        double2 c[5];
        stencil_row(o, i, j, c);
        // Each (row, column) of a front is written by one thread only; the
        // += sums couplings to neighbours that coincide (grids thinner
        // than 3 cells, explicit-stencil operators).
        F[k + k * ld] = cadd(F[k + k * ld], from_c128<T>(c[0], sigma));
        for (int d = 0; d < 4; ++d) {
            const int nl = nbr_loc[4 * s + d];
            if (nl < 0) continue;
            F[k + nl * ld] = cadd(F[k + nl * ld], from_c128<T>(c[1 + d], sigma));
            if (nl >= f.p) {
                // A[t, s] for the boundary neighbour t: t's coefficient
                // pointing back towards s.
                const int t = nbr_cell(o, i, j, d);
                double2 ct[5];
                stencil_row(o, t / o.Ny, t % o.Ny, ct);
                F[nl + k * ld] = cadd(F[nl + k * ld], from_c128<T>(ct[1 + opposite_dir(d)], sigma));
            }
        }
    }
}

// Extend-add by the parent, written once: every entry (a, b) of the
// parent's m x m block becomes the sum of the children's update-block
// entries that map onto it (inv_s[a] = child s's update-block row of parent
// row a, or -1), zero where none does, so the pool needs no clearing.  A
// CTA takes cb consecutive columns, rows fastest.  The operator's entries
// are added afterwards (k_assemble_level).
template <typename T>
__global__ void k_extend_pull(const FrontD *__restrict__ fr, const int32_t *__restrict__ inv0,
                              const int32_t *__restrict__ inv1, T *pool, int f_begin, int cb) {
    const FrontD f = fr[f_begin + blockIdx.x];
    const int b0 = blockIdx.y * cb;
    if (b0 >= f.m) return;
    const int cols = min(cb, f.m - b0), m = f.m;
    const T *U0 = nullptr, *U1 = nullptr;
    int64_t ld0 = 0, ld1 = 0;
    if (f.c0 >= 0) {
        const FrontD c = fr[f.c0];
        U0 = pool + c.f_off + (int64_t)c.p * c.ld + c.p;
        ld0 = c.ld;
    }
    if (f.c1 >= 0) {
        const FrontD c = fr[f.c1];
        U1 = pool + c.f_off + (int64_t)c.p * c.ld + c.p;
        ld1 = c.ld;
    }
    const int32_t *i0 = inv0 + f.voff, *i1 = inv1 + f.voff;
    T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    // (column, row) of entry idx = bb m + a, advanced by blockDim.x entries
    // a pass without a division per entry
    const int step_b = (int)blockDim.x / m, step_a = (int)blockDim.x - step_b * m;
    int bb = (int)threadIdx.x / m, a = (int)threadIdx.x - bb * m;
    for (int idx = threadIdx.x; idx < cols * m; idx += blockDim.x) {
        const int b = b0 + bb;
        T v = czero<T>();
        if (U0) {
            const int ia = i0[a], ib = i0[b];
            if (ia >= 0 && ib >= 0) v = U0[ia + (int64_t)ib * ld0];
        }
        if (U1) {
            const int ia = i1[a], ib = i1[b];
            if (ia >= 0 && ib >= 0) v = cadd(v, U1[ia + (int64_t)ib * ld1]);
        }
        F[a + (int64_t)b * ld] = v;
        a += step_a;
        bb += step_b;
        if (a >= m) {
            a -= m;
            ++bb;
        }
    }
}

// Row k and the boundary entries of column k of every pivot of one level
// (piv: the level's pivot variables, front by front), added to the pulled
// blocks; one thread per pivot.
template <typename T>
__device__ __forceinline__ void assemble_pivot(const OpDev &o, int sv, int k, int P, const int32_t *__restrict__ nbr_loc,
                                               const unsigned long long *maxdiag, T *D, int LD);
template <typename T>
__global__ void k_assemble_level(OpDev o, const FrontD *__restrict__ fr, const int32_t *__restrict__ piv, int count,
                                 const int32_t *__restrict__ var_front, const int32_t *__restrict__ var_loc,
                                 const int32_t *__restrict__ nbr_loc, const unsigned long long *maxdiag, T *pool) {
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
        const int sv = piv[idx];
        const FrontD f = fr[var_front[sv]];
        assemble_pivot(o, sv, var_loc[sv], f.p, nbr_loc, maxdiag, pool + f.f_off, (int)f.ld);
    }
}

// ---- dense LU of one square block in shared memory ------------------------
// k_dense_lu factors one block per front, held in shared memory (padded to a
// multiple of 16 with an identity border):
//   whole = 0: the w x w diagonal block at (k0, k0), all w pivots (the panel
//              step of a large front; w = min(64, p - k0)),
//   whole = 1: the complete m x m front with its p <= 64 pivots: L21, U12
//              and the update matrix come out of the same launch (small
//              fronts, where four launches per level would each re-read the
//              front).
// Right-looking in steps of 4 pivots: one thread factors and inverts the
// 4 x 4 diagonal block in registers, one thread per row / column forms
// L21 = A21 inv(U11) and U12 = inv(L11) A12, and all threads apply the
// rank-4 update with 4 x 4 register tiles.  The loop bodies are small and
// the same for every step, so they stay in the instruction cache (a fully
// unrolled factorization ran several times slower, fetching instructions).
// Afterwards the pivot block's inverses are completed 4 rows at a time:
//   X[B, 0:b0] = -inv(L_BB) L[B, 0:b0] X[0:b0, 0:b0]     (unit diagonals)
//   Y[0:b0, B] = -Y[0:b0, 0:b0] U[0:b0, B] inv(U_BB)
// with four threads per output column (row) splitting the sum and a quad
// shuffle to combine them.
constexpr int kStep = 4;                      // pivots per step
constexpr int kDenseMaxPiv = NB;              // pivots per launch
constexpr int kDenseThreads = 256;
constexpr size_t kDenseSmemMax = 220 * 1024;  // dynamic shared memory of one block

template <typename T>
__host__ __device__ __forceinline__ size_t dense_lu_smem(int n) {
    const int S = (n + 15) / 16 * 16;
    return (size_t)S * (S + 1) * sizeof(T);
}

// 1/b = conj(b) / |b|^2; the operands are pivots of the operator scaled to
// max|diag| = 1 and at least the static pivot threshold, so |b|^2 stays
// inside the normal range.  complex64: the hardware reciprocal estimate
// refined by one Newton-Raphson step, r' = r (2 - x r) (within an ulp of
// 1/x, and off the serial 4 x 4 step's latency compared with a
// correctly rounded reciprocal).
__device__ __forceinline__ c64 crecip_fast(c64 b) {
    const float x = fmaf(b.x, b.x, b.y * b.y);
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    const float s = r * fmaf(-x, r, 2.0f);
    return cmake<float>(b.x * s, -b.y * s);
}
__device__ __forceinline__ c128 crecip_fast(c128 b) {
    const double s = __drcp_rn(fma(b.x, b.x, b.y * b.y));
    return cmake<double>(b.x * s, -b.y * s);
}

template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst_smem, const T *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One thread: LU (no pivoting; a pivot below `tiny` in modulus is lifted
// and counted) of the kw x kw block at B (leading dimension LD), then
// inv(L) strictly below and inv(U) on and above the diagonal, in place.
template <typename T, typename R>
__device__ __forceinline__ void lu4_inv(T *B, int LD, int kw, R tiny, int *tiny_count) {
    T a[kStep][kStep];
#pragma unroll
    for (int i = 0; i < kStep; ++i)
#pragma unroll
        for (int j = 0; j < kStep; ++j)
            a[i][j] = (i < kw && j < kw) ? B[i + j * LD] : (i == j ? cone<T>() : czero<T>());
    T dinv[kStep];
    const R tiny2 = tiny * tiny;
#pragma unroll
    for (int k = 0; k < kStep; ++k) {
        if (!(cabs2(a[k][k]) >= tiny2)) {
            const R am = sqrt(cabs2(a[k][k]));
            a[k][k] = (am > R(0)) ? cmake<R>(a[k][k].x / am * tiny, a[k][k].y / am * tiny) : cmake<R>(tiny, R(0));
            atomicAdd(tiny_count, 1);
        }
        dinv[k] = crecip_fast(a[k][k]);
#pragma unroll
        for (int i = k + 1; i < kStep; ++i) {
            a[i][k] = cmul(a[i][k], dinv[k]);
#pragma unroll
            for (int j = k + 1; j < kStep; ++j) cmsub(a[i][j], a[i][k], a[k][j]);
        }
    }
    // inverses in place (no second and third 4 x 4 array: a single thread
    // runs this, and the build's register limit would otherwise spill it).
    // inv(L), unit lower, column by column from the left: X[i][j] =
    // -(L[i][j] + sum_{j<k<i} L[i][k] X[k][j]) -- columns right of j still
    // hold L
#pragma unroll
    for (int j = 0; j < kStep; ++j)
#pragma unroll
        for (int i = j + 1; i < kStep; ++i) {
            T s = a[i][j];
#pragma unroll
            for (int k = j + 1; k < i; ++k) cmac(s, a[i][k], a[k][j]);
            a[i][j] = cmake<R>(-s.x, -s.y);
        }
    // inv(U), row by row from the top: Y[i][i] = 1 / U[i][i], Y[i][j] =
    // -(sum_{i<=k<j} Y[i][k] U[k][j]) / U[j][j] -- rows below i still hold U,
    // and U[i][j] is read before it is replaced
#pragma unroll
    for (int i = 0; i < kStep; ++i) {
        a[i][i] = dinv[i];
#pragma unroll
        for (int j = i + 1; j < kStep; ++j) {
            T s = cmul(a[i][i], a[i][j]);
#pragma unroll
            for (int k = i + 1; k < j; ++k) cmac(s, a[i][k], a[k][j]);
            a[i][j] = cmul(cmake<R>(-s.x, -s.y), dinv[j]);
        }
    }
#pragma unroll
    for (int i = 0; i < kStep; ++i)
#pragma unroll
        for (int j = 0; j < kStep; ++j)
            if (i < kw && j < kw) B[i + j * LD] = a[i][j];
}

template <typename T>
__device__ __forceinline__ T shfl_c(T v, int src) {
    v.x = __shfl_sync(0xffffffffu, v.x, src);
    v.y = __shfl_sync(0xffffffffu, v.y, src);
    return v;
}

// lu4_inv by one warp: lane i + 4 j (lanes 0-15) holds entry (i, j), so no
// thread needs the 4 x 4 arrays (the register-tile build keeps its 5 x 5
// tile live across this).  The same operations in the same order as
// lu4_inv, entry by entry; the inverses go by distance from the diagonal,
// reading the factor's entries from o and the inverses' from x.  All 32
// lanes take part in every shuffle; lanes 16-31 compute nothing used.
template <typename T, typename R>
__device__ __forceinline__ void lu4_inv_warp(T *B, int LD, int kw, R tiny, int *tiny_count, int lane) {
    const int i = lane & 3, j = (lane >> 2) & 3;
    const bool mine = lane < 16 && i < kw && j < kw;
    T a = mine ? B[i + j * LD] : (i == j ? cone<T>() : czero<T>());
    const R tiny2 = tiny * tiny;
    T dj = cone<T>();  // 1 / U[j][j]
#pragma unroll
    for (int k = 0; k < kStep; ++k) {
        T piv = shfl_c(a, 5 * k);
        if (!(cabs2(piv) >= tiny2)) {
            const R am = sqrt(cabs2(piv));
            piv = (am > R(0)) ? cmake<R>(piv.x / am * tiny, piv.y / am * tiny) : cmake<R>(tiny, R(0));
            if (lane == 5 * k) {
                a = piv;
                atomicAdd(tiny_count, 1);
            }
        }
        const T d = crecip_fast(piv);
        if (j == k) dj = d;
        if (j == k && i > k) a = cmul(a, d);
        const T lik = shfl_c(a, i + 4 * k), akj = shfl_c(a, k + 4 * j);
        if (i > k && j > k) cmsub(a, lik, akj);
    }
    const T o = a;
    T x = (i == j) ? dj : o;
    // inv(L), strictly below: X[i][j] = -(L[i][j] + sum_{j<k<i} L[i][k] X[k][j])
#pragma unroll
    for (int dd = 1; dd < kStep; ++dd) {
        T s = o;
#pragma unroll
        for (int kk = 1; kk < dd; ++kk) {
            const T lik = shfl_c(o, (i + 4 * (j + kk)) & 31), xkj = shfl_c(x, ((j + kk) + 4 * j) & 31);
            if (i - j == dd) cmac(s, lik, xkj);
        }
        if (i - j == dd) x = cmake<R>(-s.x, -s.y);
    }
    // inv(U), above: Y[i][j] = -(sum_{i<=k<j} Y[i][k] U[k][j]) / U[j][j]
#pragma unroll
    for (int dd = 1; dd < kStep; ++dd) {
        const T yii = shfl_c(x, 5 * i);
        T s = cmul(yii, o);
#pragma unroll
        for (int kk = 1; kk < dd; ++kk) {
            const T yik = shfl_c(x, (i + 4 * (i + kk)) & 31), ukj = shfl_c(o, ((i + kk) + 4 * j) & 31);
            if (j - i == dd) cmac(s, yik, ukj);
        }
        if (j - i == dd) x = cmul(cmake<R>(-s.x, -s.y), dj);
    }
    if (mine) B[i + j * LD] = x;
}

// One step of the register-tile build of k_dense_lu (80-row fronts, tile
// of 5 x 5 entries a thread: rows tx + 16 i, columns ty + 16 j): the rank-kw
// update with the step's L21 columns and U12 rows read from D, on the tile
// blocks from ILO = b1 / 16 on, then the next step's panel -- columns [b1,
// b1 + n1) from row b1 down, rows [b1, b1 + n1) right of them, all inside
// block ILO -- written back to D (rt_publish).
template <int ILO, typename T, int TI>
__device__ __forceinline__ void rt_step(T (&t)[TI][TI], const T *D, int LD, int c0, int kw, int b1, int tx,
                                        int ty) {
#pragma unroll
    for (int k = 0; k < kStep; ++k) {
        if (k >= kw) break;
        T l[TI];
#pragma unroll
        for (int i = ILO; i < TI; ++i) {
            const int r = tx + 16 * i;
            l[i] = r >= b1 ? D[r + (c0 + k) * LD] : czero<T>();
        }
#pragma unroll
        for (int j = ILO; j < TI; ++j) {
            const int c = ty + 16 * j;
            const T u = c >= b1 ? D[(c0 + k) + c * LD] : czero<T>();
#pragma unroll
            for (int i = ILO; i < TI; ++i) cmsub(t[i][j], l[i], u);
        }
    }
}
template <int ILO, typename T, int TI>
__device__ __forceinline__ void rt_publish(const T (&t)[TI][TI], T *D, int LD, int b1, int n1, int tx, int ty) {
    if (ILO >= TI) return;
    const int cp = ty + 16 * ILO, rp = tx + 16 * ILO;
    if (cp >= b1 && cp < b1 + n1) {
#pragma unroll
        for (int i = ILO; i < TI; ++i) {
            const int r = tx + 16 * i;
            if (r >= b1) D[r + cp * LD] = t[i][ILO];
        }
    }
    if (rp >= b1 && rp < b1 + n1) {
#pragma unroll
        for (int j = ILO; j < TI; ++j) {
            const int c = ty + 16 * j;
            if (c >= b1 + n1) D[rp + c * LD] = t[ILO][j];
        }
    }
}

// complex64: at most 80 registers so that three CTAs share an SM (the
// leaves' fronts are latency-bound; 2 CTAs per SM ran 1.7x slower there).
// SC > 0 fixes the padded size S at compile time (every block of the launch
// has n <= SC), so that the shared-memory offsets fold into the addressing;
// SC = 0 takes S from each block.  blocked != 0 (whole fronts of the levels
// solved one warp per front) completes the inverses only inside the 16 x 16
// diagonal blocks of the pivot block and keeps L and U below / above them:
// the warp substitutions work block by block.
// Row k and the boundary entries of column k of pivot k (operator row of
// variable sv, scaled by 1/max|diag A|) into the shared-memory front D, as
// k_assemble_fronts writes them into the pool; one thread writes each entry.
template <typename T>
__device__ __forceinline__ void assemble_pivot(const OpDev &o, int sv, int k, int P, const int32_t *__restrict__ nbr_loc,
                                            const unsigned long long *maxdiag, T *D, int LD) {
    const double sigma = 1.0 / __longlong_as_double((long long)*maxdiag);
    const int i = sv / o.Ny, j = sv % o.Ny;
    double2 c[5];
    stencil_row(o, i, j, c);
    D[k + k * LD] = cadd(D[k + k * LD], from_c128<T>(c[0], sigma));
    for (int d = 0; d < 4; ++d) {
        const int nl = nbr_loc[4 * (int64_t)sv + d];
        if (nl < 0) continue;
        D[k + nl * LD] = cadd(D[k + nl * LD], from_c128<T>(c[1 + d], sigma));
        if (nl >= P) {
            const int t = nbr_cell(o, i, j, d);
            double2 ct[5];
            stencil_row(o, t / o.Ny, t % o.Ny, ct);
            D[nl + k * LD] = cadd(D[nl + k * LD], from_c128<T>(ct[1 + opposite_dir(d)], sigma));
        }
    }
}

// ASM (the leaves' builds): the front is assembled here, in shared memory,
// from the operator's rows of its pivot variables (as k_assemble_fronts
// would write them) instead of being read from the pool; a separate build
// so that the other builds keep their register allocation.
template <typename T, typename R, int SC, bool ASM>
__global__ void __launch_bounds__(kDenseThreads, sizeof(T) == 8 ? 3 : 1) k_dense_lu(const FrontD *__restrict__ fr, T *pool, int f_begin,
                                                            int k0, int whole, int blocked, R tiny, int *tiny_count,
                                                            OpDev o, const int32_t *__restrict__ asm_vars,
                                                            const int32_t *__restrict__ nbr_loc,
                                                            const unsigned long long *maxdiag) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *D = reinterpret_cast<T *>(smem_raw);
    const FrontD f = fr[f_begin + blockIdx.x];
    int n, P;
    T *G;
    if (whole) {
        n = f.m;
        P = f.p;
        G = pool + f.f_off;
    } else {
        P = min(NB, f.p - k0);
        n = P;
        G = pool + f.f_off + (int64_t)k0 * f.ld + k0;
    }
    if (P <= 0 || n <= 0) return;
    const int64_t ld = f.ld;
    const int S = SC > 0 ? SC : (n + 15) / 16 * 16, LD = S + 1, NBLK = S / 16;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (ASM) {
        for (int c = warp; c < S; c += kDenseThreads / 32)
            for (int r = lane; r < S; r += 32) D[r + c * LD] = (r == c && r >= n) ? cone<T>() : czero<T>();
        __syncthreads();
        for (int k = tid; k < P; k += kDenseThreads) assemble_pivot(o, asm_vars[f.voff + k], k, P, nbr_loc, maxdiag, D, LD);
    } else {
        for (int c = warp; c < S; c += kDenseThreads / 32)
            for (int r = lane; r < S; r += 32) {
                if (r < n && c < n)
                    cp_async_elem(D + r + c * LD, G + r + (int64_t)c * ld);
                else
                    D[r + c * LD] = (r == c) ? cone<T>() : czero<T>();
            }
        cp_async_wait_all();
    }
    __syncthreads();

    const int tx = tid & 15, ty = tid >> 4;
    // RT (complex64 blocks padded to 80 or 64: the leaves, the fronts of the
    // levels above them, the panel diagonal blocks): the trailing matrix
    // stays in registers between steps -- thread (tx, ty) owns rows tx + 16 i
    // and columns ty + 16 j, a 5 x 5 or 4 x 4 tile -- and only the next
    // step's panel column and row go back to shared memory, instead of a
    // shared-memory read-modify-write of every updated entry per step.  Same
    // operations in the same order.
    constexpr bool RT = (SC == 80 || SC == 64) && sizeof(T) == 8;
    constexpr int TI = RT ? SC / 16 : 1;
    T t[TI][TI];
    if (RT) {
#pragma unroll
        for (int i = 0; i < TI; ++i)
#pragma unroll
            for (int j = 0; j < TI; ++j) t[i][j] = D[(tx + 16 * i) + (ty + 16 * j) * LD];
    }
    for (int c0 = 0; c0 < P; c0 += kStep) {
        const int kw = min(kStep, P - c0), b1 = c0 + kw;
        if (RT) {
            if (warp == 0) lu4_inv_warp<T, R>(D + c0 + c0 * LD, LD, kw, tiny, tiny_count, lane);
        } else if (tid == 0) {
            lu4_inv<T, R>(D + c0 + c0 * LD, LD, kw, tiny, tiny_count);
        }
        __syncthreads();
        // L21 rows [b1, S): l = a inv(U11) (threads 0-127);  U12 columns
        // [b1, S): u = inv(L11) a (threads 128-255), so each warp runs one
        // of the two loops
        const int nr = S - b1;
        if (tid < kDenseThreads / 2) {
            for (int idx = b1 + tid; idx < S; idx += kDenseThreads / 2) {
                T *base = D + idx + c0 * LD;
                T v[kStep];
#pragma unroll
                for (int j = 0; j < kStep; ++j) v[j] = (j < kw) ? base[j * LD] : czero<T>();
#pragma unroll
                for (int j = 0; j < kStep; ++j) {
                    T s = czero<T>();
#pragma unroll
                    for (int k = 0; k <= j; ++k) cmac(s, v[k], D[(c0 + k) + (c0 + j) * LD]);
                    if (j < kw) base[j * LD] = s;
                }
            }
        } else {
            for (int idx = b1 + tid - kDenseThreads / 2; idx < S; idx += kDenseThreads / 2) {
                T *base = D + c0 + idx * LD;
                T v[kStep];
#pragma unroll
                for (int j = 0; j < kStep; ++j) v[j] = (j < kw) ? base[j] : czero<T>();
#pragma unroll
                for (int j = 0; j < kStep; ++j) {
                    T s = v[j];
#pragma unroll
                    for (int k = 0; k < j; ++k) cmac(s, D[(c0 + j) + (c0 + k) * LD], v[k]);
                    if (j < kw) base[j] = s;
                }
            }
        }
        (void)nr;
        __syncthreads();
        if constexpr (RT) {
            // register tiles from the first 16-block still live (b1 / 16, the
            // same on every thread) on; rows / columns of that block before
            // b1 take zero multipliers.  The update reads only column and
            // row c0 + k of D, the next panel lies in columns and rows from
            // b1 on: no barrier between the two.
            const int n1 = min(kStep, P - b1);
            switch (b1 >> 4) {
            case 0: rt_step<0>(t, D, LD, c0, kw, b1, tx, ty); rt_publish<0>(t, D, LD, b1, n1, tx, ty); break;
            case 1: rt_step<1>(t, D, LD, c0, kw, b1, tx, ty); rt_publish<1>(t, D, LD, b1, n1, tx, ty); break;
            case 2: rt_step<2>(t, D, LD, c0, kw, b1, tx, ty); rt_publish<2>(t, D, LD, b1, n1, tx, ty); break;
            case 3: rt_step<3>(t, D, LD, c0, kw, b1, tx, ty); rt_publish<3>(t, D, LD, b1, n1, tx, ty); break;
            default: rt_step<4>(t, D, LD, c0, kw, b1, tx, ty); rt_publish<4>(t, D, LD, b1, n1, tx, ty); break;
            }
            __syncthreads();
            continue;
        }
        // trailing rows / columns [b1, S) -= L21 U12 (rank kw).  Rows and
        // columns of the 16-blocks that lie before b1 take zero multipliers,
        // so their read-modify-write leaves them unchanged and the entry loop
        // needs only the block bounds, which are the same across a warp.
        const int Ilo = b1 / 16;
        for (int I0 = Ilo; I0 < NBLK; I0 += 4)
            for (int J0 = Ilo; J0 < NBLK; J0 += 4) {
                T l[4][kStep], u[kStep][4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 16 * (I0 + i) + tx;
                    const bool rl = I0 + i < NBLK && r >= b1;
#pragma unroll
                    for (int k = 0; k < kStep; ++k) l[i][k] = (rl && k < kw) ? D[r + (c0 + k) * LD] : czero<T>();
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 16 * (J0 + j) + ty;
                    const bool cl = J0 + j < NBLK && c >= b1;
#pragma unroll
                    for (int k = 0; k < kStep; ++k) u[k][j] = (cl && k < kw) ? D[(c0 + k) + c * LD] : czero<T>();
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (I0 + i < NBLK && J0 + j < NBLK) {
                            const int e = (16 * (I0 + i) + tx) + (16 * (J0 + j) + ty) * LD;
                            T acc = D[e];
#pragma unroll
                            for (int k = 0; k < kStep; ++k) cmsub(acc, l[i][k], u[k][j]);
                            D[e] = acc;
                        }
            }
        __syncthreads();
    }

    if constexpr (RT) {
        // the update matrix (rows and columns from P on) back to shared memory
#pragma unroll
        for (int i = 0; i < TI; ++i)
#pragma unroll
            for (int j = 0; j < TI; ++j) {
                const int r = tx + 16 * i, c = ty + 16 * j;
                if (r >= P && c >= P) D[r + c * LD] = t[i][j];
            }
        __syncthreads();
    }
    // off-diagonal blocks of the inverses over the P x P pivot block, 4
    // rows (columns) at a time.  Thread (col, quarter) of the lower part:
    // T[i] = L[b0+i][col] + sum_{k in (col, b0), k = quarter mod 4} L[b0+i][k] X[k][col]
    const int nb4 = (P + kStep - 1) / kStep;
    const int q = tid & 3, g = tid >> 2;  // 64 groups of four threads
    // one 4-row block b0 of both inverses; groups with act set take column
    // (row) g.  Every thread runs the shuffles and the two barriers.
    auto complete = [&](int b0, int bs, bool act) {
        T vl[kStep], vu[kStep];
        // lower: groups g < b0 take column g; upper: groups g < b0 take row g
#pragma unroll
        for (int i = 0; i < kStep; ++i) vl[i] = vu[i] = czero<T>();
        if (act) {
            const int col = g;
            for (int k = col + 1 + q; k < b0; k += 4) {
                const T x = D[k + col * LD];
#pragma unroll
                for (int i = 0; i < kStep; ++i) cmac(vl[i], D[(b0 + i) + k * LD], x);
            }
            const int row = g;
            for (int k = row + q; k < b0; k += 4) {
                const T y = D[row + k * LD];
#pragma unroll
                for (int j = 0; j < kStep; ++j) cmac(vu[j], y, D[k + (b0 + j) * LD]);
            }
        }
#pragma unroll
        for (int i = 0; i < kStep; ++i)
            for (int off = 1; off < 4; off <<= 1) {
                vl[i].x += __shfl_xor_sync(0xffffffffu, vl[i].x, off);
                vl[i].y += __shfl_xor_sync(0xffffffffu, vl[i].y, off);
                vu[i].x += __shfl_xor_sync(0xffffffffu, vu[i].x, off);
                vu[i].y += __shfl_xor_sync(0xffffffffu, vu[i].y, off);
            }
        // X[B, col] = -inv(L_BB) (L[B, col] + sum), Y[row, B] = -(sum) inv(U_BB)
        T xo[kStep], yo[kStep];
        if (act && q == 0) {
            const int col = g;
#pragma unroll
            for (int i = 0; i < kStep; ++i)
                if (i < bs) vl[i] = cadd(vl[i], D[(b0 + i) + col * LD]);
#pragma unroll
            for (int i = 0; i < kStep; ++i) {
                T s = vl[i];
#pragma unroll
                for (int k = 0; k < i; ++k) cmac(s, D[(b0 + i) + (b0 + k) * LD], vl[k]);
                xo[i] = cmake<R>(-s.x, -s.y);
            }
#pragma unroll
            for (int j = 0; j < kStep; ++j) {
                T s = czero<T>();
#pragma unroll
                for (int k = 0; k <= j; ++k) cmac(s, vu[k], D[(b0 + k) + (b0 + j) * LD]);
                yo[j] = cmake<R>(-s.x, -s.y);
            }
        }
        __syncthreads();
        if (act && q == 0) {
            const int col = g, row = g;
#pragma unroll
            for (int i = 0; i < kStep; ++i)
                if (i < bs) {
                    D[(b0 + i) + col * LD] = xo[i];
                    D[row + (b0 + i) * LD] = yo[i];
                }
        }
        __syncthreads();
    };
    if (blocked) {
        // only inside 16 x 16 diagonal blocks, which are independent: block
        // s of every 16-block at once (group g belongs to the 16-block of
        // column g, the same for the 16 groups of two warps)
        for (int sb = 1; sb < 16 / kStep; ++sb) {
            const int b0 = (g & ~15) + kStep * sb;
            complete(b0, min(kStep, P - b0), (g & 15) < kStep * sb && b0 < P);
        }
    } else {
        for (int B = 1; B < nb4; ++B) {
            const int b0 = B * kStep;
            complete(b0, min(kStep, P - b0), g < b0);
        }
    }
    for (int c = warp; c < n; c += kDenseThreads / 32)
        for (int r = lane; r < n; r += 32) G[r + (int64_t)c * ld] = D[r + c * LD];
}

// Launch k_dense_lu for blocks padded to S.  The 64-wide panel blocks and
// the leaves' 80-row fronts have their own builds (about 10% faster there;
// larger fixed sizes ran slower than the generic build).
struct LeafAsm {
    OpDev o{};
    const int32_t *vars = nullptr, *nbr_loc = nullptr;
    const unsigned long long *maxdiag = nullptr;
};

template <typename T, typename R>
void dense_lu_launch(int nfl, int S, cudaStream_t st, const FrontD *fr, T *pool, int fb, int k0, int whole,
                     int blocked, R tiny, int *tiny_count, const LeafAsm &la = LeafAsm()) {
    const size_t smem = dense_lu_smem<T>(S);
    if (la.vars) {
        if (S == 80)
            k_dense_lu<T, R, 80, true><<<nfl, kDenseThreads, smem, st>>>(
                fr, pool, fb, k0, whole, blocked, tiny, tiny_count, la.o, la.vars, la.nbr_loc, la.maxdiag);
        else
            k_dense_lu<T, R, 0, true><<<nfl, kDenseThreads, smem, st>>>(
                fr, pool, fb, k0, whole, blocked, tiny, tiny_count, la.o, la.vars, la.nbr_loc, la.maxdiag);
        return;
    }
    switch (S) {
    case 64:
        k_dense_lu<T, R, 64, false><<<nfl, kDenseThreads, smem, st>>>(fr, pool, fb, k0, whole, blocked, tiny,
                                                                      tiny_count, la.o, nullptr, nullptr, nullptr);
        break;
    case 80:
        k_dense_lu<T, R, 80, false><<<nfl, kDenseThreads, smem, st>>>(fr, pool, fb, k0, whole, blocked, tiny,
                                                                      tiny_count, la.o, nullptr, nullptr, nullptr);
        break;
    default:
        k_dense_lu<T, R, 0, false><<<nfl, kDenseThreads, smem, st>>>(fr, pool, fb, k0, whole, blocked, tiny,
                                                                     tiny_count, la.o, nullptr, nullptr, nullptr);
    }
}

enum GemmMode { SCHUR = 0, TRSM_L = 1, TRSM_U = 2 };

// Complex SIMT GEMM tile (BM x BN, K = panel width) for the three updates
// of one panel step:
//   SCHUR : F[t0:, t0:] -= L[t0:, k0:k0+w] U[k0:k0+w, t0:]
//   TRSM_L: F[t0:, k0:k0+w] = F[t0:, k0:k0+w] inv(U_kk)      (in place)
//   TRSM_U: F[k0:k0+w, t0:] = inv(L_kk) F[k0:k0+w, t0:]      (in place)
// In the in-place modes a CTA owns complete rows (TRSM_L) or columns
// (TRSM_U) of its output and reads all of them before writing.
// QA x QB 16-row / 16-column groups per thread: the tile is (16 QA) x (16 QB).
template <typename T, typename R, int MODE, int QA = 4, int QB = 4>
__device__ __forceinline__ void gemm_tile(const FrontD *__restrict__ fr, T *pool, int f_begin, int k0, int ytile,
                                          int ztile, T (*As)[BM + 1], T (*Bs)[BN + 1], uint8_t *bpack = nullptr) {
    const FrontD f = fr[f_begin + blockIdx.x];
    const int w = min(NB, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w;
    const int m = f.m;
    constexpr int TM = 16 * QA, TN = 16 * QB;
    int rbase, cbase, rend, cend;
    if (MODE == SCHUR) {
        rbase = t0 + ytile * TM; cbase = t0 + ztile * TN; rend = m; cend = m;
    } else if (MODE == TRSM_L) {
        rbase = t0 + ytile * TM; cbase = k0; rend = m; cend = t0;
    } else {
        rbase = k0; cbase = t0 + ztile * TN; rend = t0; cend = m;
    }
    if (rbase >= rend || cbase >= cend) return;
    T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    T acc[QA][QB];
#pragma unroll
    for (int a = 0; a < QA; ++a)
#pragma unroll
        for (int b = 0; b < QB; ++b) acc[a][b] = czero<T>();

    // The A and B elements of K chunk kc + BK load into registers while
    // chunk kc is multiplied out of shared memory.
    auto load_a = [&](int kc, int q) -> T {
        const int idx = tid + 256 * q;
        const int rr = idx % TM, kk = idx / TM;
        const int r = rbase + rr, kg = kc + kk;
        T v = czero<T>();
        if (r < rend && kg < w) {
            if (MODE == TRSM_U) {
                // unit lower inv(L_kk): rows are k0 + rr
                const int lr = rr;
                if (kg < lr) v = F[(k0 + lr) + (int64_t)(k0 + kg) * ld];
                else if (kg == lr) v = cone<T>();
            } else {
                v = F[r + (int64_t)(k0 + kg) * ld];
            }
        }
        return v;
    };
    auto load_b = [&](int kc, int q) -> T {
        const int idx = tid + 256 * q;
        const int kk = idx % BK, cc = idx / BK;
        const int c = cbase + cc, kg = kc + kk;
        T v = czero<T>();
        if (c < cend && kg < w) {
            if (MODE == TRSM_L) {
                // upper inv(U_kk): cols are k0 + (c - k0)
                const int uc = c - k0;
                if (kg <= uc) v = F[(k0 + kg) + (int64_t)c * ld];
            } else {
                v = F[(k0 + kg) + (int64_t)c * ld];
            }
        }
        return v;
    };
    T pa[QA], pb[QB];
#pragma unroll
    for (int q = 0; q < QA; ++q) pa[q] = load_a(0, q);
#pragma unroll
    for (int q = 0; q < QB; ++q) pb[q] = load_b(0, q);
    for (int kc = 0; kc < w; kc += BK) {
#pragma unroll
        for (int q = 0; q < QA; ++q) {
            const int idx = tid + 256 * q;
            As[idx / TM][idx % TM] = pa[q];
        }
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int idx = tid + 256 * q;
            Bs[idx % BK][idx / BK] = pb[q];
        }
        __syncthreads();
        if (kc + BK < w) {
#pragma unroll
            for (int q = 0; q < QA; ++q) pa[q] = load_a(kc + BK, q);
#pragma unroll
            for (int q = 0; q < QB; ++q) pb[q] = load_b(kc + BK, q);
        }
        // the triangular inverses are zero below (inv(U), TRSM_L) or above
        // (inv(L), TRSM_U) their diagonal: K chunk kc adds nothing to the
        // output columns (rows) of the 16-blocks before it
        const int kcb = kc / 16;
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[QA], b[QB];
#pragma unroll
            for (int q = 0; q < QA; ++q) a[q] = As[kk][ty + 16 * q];
#pragma unroll
            for (int q = 0; q < QB; ++q) b[q] = Bs[kk][tx + 16 * q];
#pragma unroll
            for (int qa = 0; qa < QA; ++qa) {
                if (MODE == TRSM_U && qa < kcb) continue;
#pragma unroll
                for (int qb = 0; qb < QB; ++qb) {
                    if (MODE == TRSM_L && qb < kcb) continue;
                    cmac(acc[qa][qb], a[qa], b[qb]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int qa = 0; qa < QA; ++qa) {
        const int r = rbase + ty + 16 * qa;
        if (r >= rend) continue;
#pragma unroll
        for (int qb = 0; qb < QB; ++qb) {
            const int c = cbase + tx + 16 * qb;
            if (c >= cend) continue;
            T &dst = F[r + (int64_t)c * ld];
            if (MODE == SCHUR) dst = csub(dst, acc[qa][qb]);
            else dst = acc[qa][qb];
        }
    }
    if constexpr (MODE == TRSM_U && std::is_same<T, c64>::value) {
        // tensor-core levels: the U panel also goes straight into its packed
        // B'' tiles (hi/lo TF32), zero outside the panel and the front
        if (bpack) {
            const int cts = (m - t0 + kTileNc - 1) / kTileNc;
#pragma unroll
            for (int qa = 0; qa < QA; ++qa) {
                const int r = rbase + ty + 16 * qa, l = r - k0;
#pragma unroll
                for (int qb = 0; qb < QB; ++qb) {
                    const int c = cbase + tx + 16 * qb, cc = c - t0, ct = cc / kTileNc;
                    if (ct >= cts) continue;
                    const c64 v = (r < rend && c < cend) ? acc[qa][qb] : czero<c64>();
                    uint8_t *hi = bpack + (size_t)ct * 2 * kBTileBytes;
                    tc_store_b(hi, hi + kBTileBytes, l, cc - ct * kTileNc, v);
                }
            }
            // a narrow tile (panels of at most 32 pivots) covers panel rows
            // [0, 16 QA); the packed rows after it are zero too
#pragma unroll
            for (int qa = QA; qa < 4; ++qa) {
                const int l = ty + 16 * qa;
#pragma unroll
                for (int qb = 0; qb < QB; ++qb) {
                    const int c = cbase + tx + 16 * qb, cc = c - t0, ct = cc / kTileNc;
                    if (ct >= cts) continue;
                    uint8_t *hi = bpack + (size_t)ct * 2 * kBTileBytes;
                    tc_store_b(hi, hi + kBTileBytes, l, cc - ct * kTileNc, czero<c64>());
                }
            }
        }
    }
}

template <typename T, typename R>
__global__ void __launch_bounds__(256) k_schur_simt(const FrontD *__restrict__ fr, T *pool, int f_begin, int k0) {
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    gemm_tile<T, R, SCHUR>(fr, pool, f_begin, k0, blockIdx.y, blockIdx.z, As, Bs);
}

// Both triangular updates of a panel step in one launch: blockIdx.z = 0
// forms L (row tile blockIdx.y), blockIdx.z = 1 forms U (column tile
// blockIdx.y) and, on tensor-core levels (tcf != NULL), its packed tiles.
// HALF: 32-row (L) / 32-column (U) tiles, twice the CTAs, for levels with
// few fronts whose triangular updates would not fill the GPU.
// Q = 4, 2 or 1: output tiles of 16 Q rows (L21) / 16 Q columns (U12).
// QW = 4 or 2: the panel's side of the tiles, 64 or (panels of at most 32
// pivots: the single-panel fronts of the levels above the leaves) 32 wide,
// so that those panels compute no zero columns (rows).
template <typename T, typename R, int Q, int QW>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 3 : 1) k_trsm_panel(const FrontD *__restrict__ fr, T *pool, int f_begin, int k0,
                                                    const TcFront *__restrict__ tcf, uint8_t *scratch) {
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    if (blockIdx.z == 0) {
        gemm_tile<T, R, TRSM_L, Q, QW>(fr, pool, f_begin, k0, blockIdx.y, 0, As, Bs);
    } else {
        uint8_t *bpack = tcf ? scratch + tcf[f_begin + blockIdx.x].b_off : nullptr;
        gemm_tile<T, R, TRSM_U, QW, Q>(fr, pool, f_begin, k0, 0, blockIdx.y, As, Bs, bpack);
    }
}

// Both triangular updates of panel k0 for the fronts of a level (trail: an
// upper bound of m - t0).  Half-height tiles while the level would launch
// fewer than 1024 CTAs, quarter-height ones below 256 (the last panels of the
// few large fronts near the root, on the factorization's critical path).
template <typename T, typename R, int QW>
void trsm_launch_w(int nfl, int trail, cudaStream_t st, const FrontD *fr, T *pool, int fb, int k0,
                   const TcFront *tcf, uint8_t *scratch) {
    const int tiles = (trail + BM - 1) / BM;
    if (nfl * tiles * 2 < 256) {
        const int t4 = (trail + BM / 4 - 1) / (BM / 4);
        k_trsm_panel<T, R, 1, QW><<<dim3(nfl, t4, 2), 256, 0, st>>>(fr, pool, fb, k0, tcf, scratch);
    } else if (nfl * tiles * 2 < 1024) {
        const int t2 = (trail + BM / 2 - 1) / (BM / 2);
        k_trsm_panel<T, R, 2, QW><<<dim3(nfl, t2, 2), 256, 0, st>>>(fr, pool, fb, k0, tcf, scratch);
    } else {
        k_trsm_panel<T, R, 4, QW><<<dim3(nfl, tiles, 2), 256, 0, st>>>(fr, pool, fb, k0, tcf, scratch);
    }
}
// maxw: the level's widest panel at k0 (min(64, max p - k0))
template <typename T, typename R>
void trsm_launch(int nfl, int trail, int maxw, cudaStream_t st, const FrontD *fr, T *pool, int fb, int k0,
                 const TcFront *tcf, uint8_t *scratch) {
    if (maxw <= NB / 2)
        trsm_launch_w<T, R, 2>(nfl, trail, st, fr, pool, fb, k0, tcf, scratch);
    else
        trsm_launch_w<T, R, 4>(nfl, trail, st, fr, pool, fb, k0, tcf, scratch);
}

// ---- solve ------------------------------------------------------------------
// Workspace layout: W[rhs * sum_m + voff + k] (front-local vectors), Y the
// same shape (forward solution of the pivot rows).

// Forward, step 1: rhs entries of the pivots and the children's updates.
template <typename T>
__global__ void k_fwd_gather(const FrontD *__restrict__ fr, const int32_t *__restrict__ vars,
                             const int32_t *__restrict__ relmap, const double2 *__restrict__ b,
                             const double *__restrict__ s_in, T *W, int64_t sum_m, int64_t n,
                             int nrhs, int f_begin) {
    const FrontD f = fr[f_begin + blockIdx.x];
    const int32_t *v = vars + f.voff;
    for (int r = 0; r < nrhs; ++r) {
        T *w = W + r * sum_m + f.voff;
        const double s = s_in[r];
        for (int k = threadIdx.x; k < f.m; k += blockDim.x)
            w[k] = (k < f.p) ? from_c128<T>(b[r * n + v[k]], s) : czero<T>();
    }
    __syncthreads();
    for (int slot = 0; slot < 2; ++slot) {
        const int c = slot ? f.c1 : f.c0;
        if (c < 0) continue;
        const FrontD ch = fr[c];
        const int mu = ch.m - ch.p;
        const int32_t *rm = relmap + ch.voff + ch.p;
        for (int r = 0; r < nrhs; ++r) {
            T *w = W + r * sum_m + f.voff;
            const T *wc = W + r * sum_m + ch.voff + ch.p;
            for (int a = threadIdx.x; a < mu; a += blockDim.x) w[rm[a]] = cadd(w[rm[a]], wc[a]);
        }
        __syncthreads();
    }
}

// Forward gather of one front into ws (nrhs x ld_ws): w = s_in b on the
// pivots (zero on the boundary), plus child 0's update, plus child 1's, added in
// that order; inv0 / inv1 give each of the front's rows its row in the
// children's update blocks (or -1).  Threads t, t + nt, ... of the caller.
template <typename T>
__device__ __forceinline__ void gather_front(const FrontD *__restrict__ fr, const FrontD &f,
                                             const int32_t *__restrict__ v, const int32_t *__restrict__ inv0,
                                             const int32_t *__restrict__ inv1, const double2 *__restrict__ b,
                                             const double *__restrict__ s_in, const T *W, int64_t sum_m, int64_t n,
                                             int nrhs, T *ws, int ld_ws, int t,
                                             int nt) {
    const int64_t u0 = f.c0 >= 0 ? (int64_t)fr[f.c0].voff + fr[f.c0].p : 0;
    const int64_t u1 = f.c1 >= 0 ? (int64_t)fr[f.c1].voff + fr[f.c1].p : 0;
    for (int k = t; k < f.m; k += nt) {
        const int a0 = f.c0 >= 0 ? inv0[f.voff + k] : -1, a1 = f.c1 >= 0 ? inv1[f.voff + k] : -1;
        const int var = k < f.p ? v[k] : 0;
        for (int r = 0; r < nrhs; ++r) {
            T w = (k < f.p) ? from_c128<T>(b[r * n + var], s_in[r]) : czero<T>();
            if (a0 >= 0) w = cadd(w, W[r * sum_m + u0 + a0]);
            if (a1 >= 0) w = cadd(w, W[r * sum_m + u1 + a1]);
            ws[r * ld_ws + k] = w;
        }
    }
}

// ---- substitutions of levels whose fronts have at most 64 pivots --------------
// One CTA per front does the whole step of a direction (the gather, the
// triangular product with the stored inverse and the update rows), instead
// of a gather launch plus one launch per panel.  Products are taken 32 rows
// at a time: the rows go to consecutive lanes, so each load instruction
// reads 32 consecutive entries of a column of the column-major front, and
// eight thread groups split every sum by column (eight loads in flight per
// row) before meeting in shared memory.
constexpr int kSmallThreads = 256;
constexpr int kSmallMaxM = 2048;  // fronts up to this size use the one-launch steps
constexpr size_t kSmallSmemMax = 200 * 1024;
constexpr int kSmallGroups = kSmallThreads / 32;

template <typename T>
__host__ __device__ __forceinline__ size_t small_smem_bytes(int nrhs, int maxm) {
    return ((size_t)(nrhs + 1) * maxm + kSmallThreads) * sizeof(T);
}

// res[i] = sum_t F[row0 + i, t] v[t] for i < nrows, with t in [lo, hi)
// (RANGE = 0), t < row0 + i (RANGE = 1) or t in [row0 + i, hi) (RANGE = 2).
template <typename T, int RANGE>
__device__ __forceinline__ void rows_dot(const T *F, int64_t ld, int row0, int nrows, int lo, int hi, const T *v,
                                         T *part, T *res) {
    const int rr = threadIdx.x & 31, g = threadIdx.x >> 5;
    for (int c = 0; c < nrows; c += 32) {
        const int i = c + rr, row = row0 + i;
        T s = czero<T>();
        if (i < nrows) {
            const int a = (RANGE == 2) ? row : (RANGE == 1 ? 0 : lo);
            const int e = (RANGE == 1) ? row : hi;
            for (int t = a + g; t < e; t += kSmallGroups) cmac(s, F[row + (int64_t)t * ld], v[t]);
        }
        part[g * 32 + rr] = s;
        __syncthreads();
        if (g == 0 && i < nrows) {
            T tot = part[rr];
#pragma unroll
            for (int q = 1; q < kSmallGroups; ++q) tot = cadd(tot, part[q * 32 + rr]);
            res[i] = tot;
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(kSmallThreads)
    k_fwd_small(const FrontD *__restrict__ fr, const int32_t *__restrict__ vars, const int32_t *__restrict__ inv0,
                const int32_t *__restrict__ inv1,
                const T *__restrict__ pool, const double2 *__restrict__ b, const double *__restrict__ s_in, T *W,
                T *Y, int64_t sum_m, int64_t n, int nrhs, int f_begin, int maxm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *ws = reinterpret_cast<T *>(smem_raw);   // [rhs][maxm]
    T *tmp = ws + (size_t)nrhs * maxm;          // [maxm]
    T *part = tmp + maxm;                       // [groups][32]
    const FrontD f = fr[f_begin + blockIdx.x];
    const int32_t *v = vars + f.voff;
    const int tid = threadIdx.x;
    gather_front(fr, f, v, inv0, inv1, b, s_in, W, sum_m, n, nrhs, ws, maxm, tid, blockDim.x);
    __syncthreads();
    const T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    for (int r = 0; r < nrhs; ++r) {
        T *w = ws + r * maxm;
        // y = inv(L11) w_P (unit diagonal): y_i = w_i + sum_{t<i} invL[i][t] w_t
        rows_dot<T, 1>(F, ld, 0, f.p, 0, 0, w, part, tmp);
        for (int i = tid; i < f.p; i += blockDim.x) {
            const T y = cadd(w[i], tmp[i]);
            w[i] = y;
            Y[r * sum_m + f.voff + i] = y;
        }
        __syncthreads();
        // update rows: w_B -= L21 y
        rows_dot<T, 0>(F, ld, f.p, f.m - f.p, 0, f.p, w, part, tmp);
        for (int i = tid; i < f.m - f.p; i += blockDim.x)
            W[r * sum_m + f.voff + f.p + i] = csub(w[f.p + i], tmp[i]);
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(kSmallThreads)
    k_bwd_small(const FrontD *__restrict__ fr, const int32_t *__restrict__ vars, const T *__restrict__ pool,
                const T *__restrict__ Y, double2 *x, int64_t sum_m, int64_t n, int nrhs, int f_begin, int maxm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);  // [rhs][maxm]: pivots then x_B
    T *tmp = xs + (size_t)nrhs * maxm;
    T *part = tmp + maxm;
    const FrontD f = fr[f_begin + blockIdx.x];
    const int32_t *v = vars + f.voff;
    const int tid = threadIdx.x;
    for (int r = 0; r < nrhs; ++r)
        for (int k = f.p + tid; k < f.m; k += blockDim.x) xs[r * maxm + k] = from_c128<T>(x[r * n + v[k]], 1.0);
    __syncthreads();
    const T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    for (int r = 0; r < nrhs; ++r) {
        T *xr = xs + r * maxm;
        // acc = y - U12 x_B
        rows_dot<T, 0>(F, ld, 0, f.p, f.p, f.m, xr, part, tmp);
        for (int i = tid; i < f.p; i += blockDim.x) xr[i] = csub(Y[r * sum_m + f.voff + i], tmp[i]);
        __syncthreads();
        // x_P = inv(U11) acc: x_i = sum_{t>=i} invU[i][t] acc_t
        rows_dot<T, 2>(F, ld, 0, f.p, 0, f.p, xr, part, tmp);
        for (int i = tid; i < f.p; i += blockDim.x) x[r * n + v[i]] = to_c128(tmp[i], 1.0);
        __syncthreads();
    }
}

// Levels of small fronts (m <= 128): one warp per front, eight fronts per
// CTA.  A lane owns rows (lane, lane + 32, ...) of the front and streams
// the column-major entries of its rows column by column (32 consecutive
// entries per load instruction, several columns in flight), with the
// vectors in the warp's shared memory; no block barrier is involved.
constexpr int kWarpMaxM = 128;
constexpr int kWarpFronts = 8;

template <typename T>
__host__ __device__ __forceinline__ size_t warp_smem_bytes(int nrhs, int maxm) {
    return (size_t)kWarpFronts * nrhs * maxm * sizeof(T);
}

template <typename T>
__device__ __forceinline__ T pick4(const T (&a)[4], int k) {
    return k == 0 ? a[0] : k == 1 ? a[1] : k == 2 ? a[2] : a[3];
}

// Blocked forward substitution of one front by one warp (blocked pivot-
// block format): w (shared, length m) holds the gathered right-hand side;
// the pivot rows R_k = lane + 32 k (k < 2, p <= 64) accumulate in acc[k].
// Per 16-block I of the pivots: the block's accumulated values go through
// w, each block lane forms y_r = acc_r + sum_{c0 <= c < r} inv(L_II)[r, c]
// acc_c, and the pivot rows of later blocks take acc_R -= L[R, I] y_I.  On
// return w[0, p) holds y (the update rows are formed afterwards in one pass
// over L21, as with the full inverse).
template <typename T>
__device__ __forceinline__ void warp_fwd_blocked(const T *F, int64_t ld, int p, T *w, int lane) {
    T acc[4];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int R = lane + 32 * k;
        acc[k] = R < p ? w[R] : czero<T>();
    }
    acc[2] = acc[3] = czero<T>();
    for (int c0 = 0; c0 < p; c0 += 16) {
        const int cw = min(16, p - c0), kI = c0 >> 5, l0 = c0 & 31;
        const bool inb = lane >= l0 && lane < l0 + cw;
        const int r = c0 + lane - l0;
        if (inb) w[r] = pick4(acc, kI);
        __syncwarp();
        T y = czero<T>();
        if (inb) {
            y = w[r];
#pragma unroll
            for (int j = 0; j < 15; ++j)
                if (c0 + j < r) cmac(y, F[r + (int64_t)(c0 + j) * ld], w[c0 + j]);
        }
        __syncwarp();
        if (inb) w[r] = y;
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int R = lane + 32 * k;
            if (k == kI && inb) acc[k] = y;
            if (R >= c0 + cw && R < p) {
                T sum = czero<T>();
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (j < cw) cmac(sum, F[R + (int64_t)(c0 + j) * ld], w[c0 + j]);
                acc[k] = csub(acc[k], sum);
            }
        }
    }
    __syncwarp();
}

// Blocked backward substitution (blocked format): on entry acc[k] holds
// y_R - U12[R, :] x_B for the pivot rows R = lane + 32 k < p.  Per 16-block
// I from the last: x_I = inv(U_II) acc_I through xr, then every earlier
// pivot row takes acc_R -= U[R, I] x_I.  On return xr[0, p) holds x_P.
template <typename T>
__device__ __forceinline__ void warp_bwd_blocked(const T *F, int64_t ld, int p, T *xr, int lane, T (&acc)[4]) {
    for (int c0 = (p - 1) & ~15; c0 >= 0; c0 -= 16) {
        const int cw = min(16, p - c0), kI = c0 >> 5, l0 = c0 & 31;
        const bool inb = lane >= l0 && lane < l0 + cw;
        const int r = c0 + lane - l0;
        if (inb) xr[r] = pick4(acc, kI);
        __syncwarp();
        T xv = czero<T>();
        if (inb) {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (j < cw && c0 + j >= r) cmac(xv, F[r + (int64_t)(c0 + j) * ld], xr[c0 + j]);
        }
        __syncwarp();
        if (inb) xr[r] = xv;
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int R = lane + 32 * k;
            if (R < c0) {
                T sum = czero<T>();
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (j < cw) cmac(sum, F[R + (int64_t)(c0 + j) * ld], xr[c0 + j]);
                acc[k] = csub(acc[k], sum);
            }
        }
    }
    __syncwarp();
}

// complex64: at most 48 (forward) / 40 (backward) registers, so that 40 / 48
// warps stay resident on an SM -- the passes wait on their loads (long
// scoreboard), and more warps keep more of them in flight.
template <typename T>
__global__ void __launch_bounds__(32 * kWarpFronts, sizeof(T) == 8 ? 5 : 4)
    k_fwd_warp(const FrontD *__restrict__ fr, const int32_t *__restrict__ vars, const int32_t *__restrict__ inv0,
               const int32_t *__restrict__ inv1,
               const T *__restrict__ pool, const double2 *__restrict__ b, const double *__restrict__ s_in, T *W,
               T *Y, int64_t sum_m, int64_t n, int nrhs, int f_begin, int nfl, int maxm, int blocked) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int fi = blockIdx.x * kWarpFronts + warp;
    if (fi >= nfl) return;
    T *ws = reinterpret_cast<T *>(smem_raw) + (size_t)warp * nrhs * maxm;
    const FrontD f = fr[f_begin + fi];
    const int32_t *v = vars + f.voff;
    const int p = f.p, m = f.m;
    gather_front(fr, f, v, inv0, inv1, b, s_in, W, sum_m, n, nrhs, ws, maxm, lane, 32);
    __syncwarp();
    const T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    const int r0 = lane, r1 = lane + 32;
    for (int r = 0; r < nrhs; ++r) {
        T *w = ws + r * maxm;
        if (blocked) {
            warp_fwd_blocked(F, ld, p, w, lane);
            if (r0 < p) Y[r * sum_m + f.voff + r0] = w[r0];
            if (r1 < p) Y[r * sum_m + f.voff + r1] = w[r1];
        }
        // y = inv(L11) w_P: y_i = w_i + sum_{t<i} invL[i][t] w_t (rows r0, r1 < p <= 64)
        T a0 = czero<T>(), a1 = czero<T>();
        if (!blocked) {
#pragma unroll 8
            for (int t = 0; t < p; ++t) {
                const T wt = w[t];
                if (t < r0) cmac(a0, F[r0 + (int64_t)t * ld], wt);
                if (t < r1 && r1 < p) cmac(a1, F[r1 + (int64_t)t * ld], wt);
            }
            __syncwarp();
            if (r0 < p) {
                const T y = cadd(w[r0], a0);
                w[r0] = y;
                Y[r * sum_m + f.voff + r0] = y;
            }
            if (r1 < p) {
                const T y = cadd(w[r1], a1);
                w[r1] = y;
                Y[r * sum_m + f.voff + r1] = y;
            }
            __syncwarp();
        }
        // update rows: w_B -= L21 y
        for (int rb = p; rb < m; rb += 32) {
            const int row = rb + lane;
            T a = czero<T>();
            if (row < m) {
#pragma unroll 8
                for (int t = 0; t < p; ++t) cmac(a, F[row + (int64_t)t * ld], w[t]);
                W[r * sum_m + f.voff + row] = csub(w[row], a);
            }
        }
        __syncwarp();
    }
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarpFronts, sizeof(T) == 8 ? 6 : 4)
    k_bwd_warp(const FrontD *__restrict__ fr, const int32_t *__restrict__ vars, const T *__restrict__ pool,
               const T *__restrict__ Y, double2 *x, int64_t sum_m, int64_t n, int nrhs, int f_begin, int nfl,
               int maxm, int blocked) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int fi = blockIdx.x * kWarpFronts + warp;
    if (fi >= nfl) return;
    T *xs = reinterpret_cast<T *>(smem_raw) + (size_t)warp * nrhs * maxm;
    const FrontD f = fr[f_begin + fi];
    const int32_t *v = vars + f.voff;
    const int p = f.p, m = f.m;
    for (int r = 0; r < nrhs; ++r)
        for (int k = p + lane; k < m; k += 32) xs[r * maxm + k] = from_c128<T>(x[r * n + v[k]], 1.0);
    __syncwarp();
    const T *F = pool + f.f_off;
    const int64_t ld = f.ld;
    const int r0 = lane, r1 = lane + 32;
    for (int r = 0; r < nrhs; ++r) {
        T *xr = xs + r * maxm;
        // acc = y - U12 x_B
        T a0 = czero<T>(), a1 = czero<T>();
#pragma unroll 8
        for (int c = p; c < m; ++c) {
            const T xc = xr[c];
            if (r0 < p) cmac(a0, F[r0 + (int64_t)c * ld], xc);
            if (r1 < p) cmac(a1, F[r1 + (int64_t)c * ld], xc);
        }
        if (blocked) {
            T acc[4];
            acc[0] = r0 < p ? csub(Y[r * sum_m + f.voff + r0], a0) : czero<T>();
            acc[1] = r1 < p ? csub(Y[r * sum_m + f.voff + r1], a1) : czero<T>();
            acc[2] = acc[3] = czero<T>();
            warp_bwd_blocked(F, ld, p, xr, lane, acc);
            if (r0 < p) x[r * n + v[r0]] = to_c128(xr[r0], 1.0);
            if (r1 < p) x[r * n + v[r1]] = to_c128(xr[r1], 1.0);
            __syncwarp();
            continue;
        }
        if (r0 < p) xr[r0] = csub(Y[r * sum_m + f.voff + r0], a0);
        if (r1 < p) xr[r1] = csub(Y[r * sum_m + f.voff + r1], a1);
        __syncwarp();
        // x_P = inv(U11) acc: x_i = sum_{t>=i} invU[i][t] acc_t
        T s0 = czero<T>(), s1 = czero<T>();
#pragma unroll 8
        for (int t = 0; t < p; ++t) {
            const T at = xr[t];
            if (t >= r0) cmac(s0, F[r0 + (int64_t)t * ld], at);
            if (t >= r1 && r1 < p) cmac(s1, F[r1 + (int64_t)t * ld], at);
        }
        if (r0 < p) x[r * n + v[r0]] = to_c128(s0, 1.0);
        if (r1 < p) x[r * n + v[r1]] = to_c128(s1, 1.0);
        __syncwarp();
    }
}

// ---- shared panel-step helpers of the triangular solves ------------------------
// Shared memory of one panel step: the w x w diagonal block (only its
// triangle), the input vector block and the result block, staged with
// coalesced loads so that the dependent triangular product runs out of
// shared memory instead of waiting on a global load per term.
template <typename T>
__host__ __device__ __forceinline__ size_t panel_smem_bytes(int nrhs) {
    return (size_t)(NB * NB + 2 * nrhs * NB) * sizeof(T);
}

// out = inv(L_kk) v (UPPER = false: unit lower inverse stored strictly below
// the diagonal) or out = inv(U_kk) v (UPPER = true: on and above).  v is
// read from vin_g (per rhs stride vstride); result left in sm (returned).
template <typename T, typename R, bool UPPER>
__device__ __forceinline__ T *panel_diag_apply(const T *F, int64_t ld, int k0, int w, const T *vin_g,
                                               int64_t vstride, int nrhs, T *sm) {
    T *Ds = sm, *vin = sm + NB * NB, *out = vin + nrhs * NB;
    const int tid = threadIdx.x;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        const bool need = UPPER ? (r <= c) : (r > c);
        Ds[r + c * NB] = need ? F[(k0 + r) + (int64_t)(k0 + c) * ld] : czero<T>();
    }
    for (int idx = tid; idx < nrhs * w; idx += blockDim.x) {
        const int r = idx / w, i = idx % w;
        vin[r * NB + i] = vin_g[r * vstride + k0 + i];
    }
    __syncthreads();
    for (int idx = tid; idx < nrhs * w; idx += blockDim.x) {
        const int r = idx / w, row = idx % w;
        const T *vr = vin + r * NB;
        T acc;
        if (UPPER) {
            acc = czero<T>();
            for (int t = row; t < w; ++t) cmac(acc, Ds[row + t * NB], vr[t]);
        } else {
            acc = vr[row];
            for (int t = 0; t < row; ++t) cmac(acc, Ds[row + t * NB], vr[t]);
        }
        out[r * NB + row] = acc;
    }
    __syncthreads();
    return out;
}

// Row-block update of a panel step: dst[row] -= F[row, k0:k0+w] y for the
// kItemRows rows starting at rbase (rows >= rend skipped).  Four threads
// share a row, each with 16 independent column loads in flight, and the
// four partial sums meet through warp shuffles: the update is bound by how
// many loads are outstanding, not by arithmetic.
constexpr int kItemRows = 64;
template <typename T>
__device__ __forceinline__ void panel_rows_update(const T *F, int64_t ld, int k0, int w, int rbase, int rend,
                                                  const T *y, int nrhs, T *dst, int64_t dstride) {
    const int rr = threadIdx.x >> 2, q = threadIdx.x & 3;
    const int row = rbase + rr;
    const bool live = row < rend;
    T acc[8];
    for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
    if (live) {
        const T *Fr = F + row + (int64_t)(k0 + 16 * q) * ld;
        const int t0 = 16 * q;
        if (t0 + 16 <= w) {
            T a[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) a[i] = Fr[(int64_t)i * ld];
            for (int r = 0; r < nrhs; ++r) {
                const T *yr = y + r * NB + t0;
#pragma unroll
                for (int i = 0; i < 16; ++i) cmac(acc[r], a[i], yr[i]);
            }
        } else {
            for (int i = 0; t0 + i < w; ++i) {
                const T a = Fr[(int64_t)i * ld];
                for (int r = 0; r < nrhs; ++r) cmac(acc[r], a, y[r * NB + t0 + i]);
            }
        }
    }
    for (int r = 0; r < nrhs; ++r) {
        for (int off = 1; off < 4; off <<= 1) {
            acc[r].x += __shfl_xor_sync(0xffffffffu, acc[r].x, off);
            acc[r].y += __shfl_xor_sync(0xffffffffu, acc[r].y, off);
        }
        if (live && q == 0) {
            T &d = dst[r * dstride + row];
            d = csub(d, acc[r]);
        }
    }
}

// Row-block product for the backward opener: acc[rhs] = sum over columns
// [c0, c0+cn) of F[row, c] xs[rhs][c - c0] (xs in shared memory, row
// stride kRowsPerCta), four threads per row as in panel_rows_update.
template <typename T, int N>
__device__ __forceinline__ void opener_rows_product(const T *F, int64_t ld, int row, bool live, int c0, int cn,
                                                    const T *xs, int nrhs, T (&acc)[N]) {
    const int q = threadIdx.x & 3;
    if (live) {
        for (int cb = 16 * q; cb < cn; cb += 64) {
            const T *Fr = F + row + (int64_t)(c0 + cb) * ld;
            const int len = min(16, cn - cb);
            if (len == 16) {
                T a[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) a[i] = Fr[(int64_t)i * ld];
                for (int r = 0; r < nrhs; ++r) {
                    const T *xr = xs + r * kRowsPerCta + cb;
#pragma unroll
                    for (int i = 0; i < 16; ++i) cmac(acc[r], a[i], xr[i]);
                }
            } else {
                for (int i = 0; i < len; ++i) {
                    const T a = Fr[(int64_t)i * ld];
                    for (int r = 0; r < nrhs; ++r) cmac(acc[r], a, xs[r * kRowsPerCta + cb + i]);
                }
            }
        }
    }
}

template <typename T, int N>
__device__ __forceinline__ void quad_reduce(T (&acc)[N], int nrhs) {
    for (int r = 0; r < nrhs; ++r)
        for (int off = 1; off < 4; off <<= 1) {
            acc[r].x += __shfl_xor_sync(0xffffffffu, acc[r].x, off);
            acc[r].y += __shfl_xor_sync(0xffffffffu, acc[r].y, off);
        }
}

// Forward, one panel: y_k = inv(L_kk) w_k (every CTA of the front computes
// it; CTA 0 stores it to Y), then w[t0:m] -= L[t0:m, k] y_k.
template <typename T, typename R>
__global__ void k_fwd_panel(const FrontD *__restrict__ fr, const T *__restrict__ pool, T *W, T *Y,
                            int64_t sum_m, int nrhs, int f_begin, int k0) {
    extern __shared__ unsigned char smem_raw[];
    const FrontD f = fr[f_begin + blockIdx.x];
    const int w = min(NB, f.p - k0);
    if (w <= 0) return;
    const int t0 = k0 + w;
    const int rbase = t0 + blockIdx.y * kItemRows;
    if (blockIdx.y > 0 && rbase >= f.m) return;
    const T *F = pool + f.f_off;
    const int tid = threadIdx.x;
    T *yk = panel_diag_apply<T, R, false>(F, f.ld, k0, w, W + f.voff, sum_m, nrhs,
                                          reinterpret_cast<T *>(smem_raw));
    if (blockIdx.y == 0)
        for (int idx = tid; idx < nrhs * w; idx += blockDim.x) {
            const int r = idx / w, row = idx % w;
            Y[r * sum_m + f.voff + k0 + row] = yk[r * NB + row];
        }
    panel_rows_update(F, f.ld, k0, w, rbase, f.m, yk, nrhs, W + f.voff, sum_m);
}

// Backward, step 1: acc[0:p] = y[0:p] - U[0:p, p:m] x_B, x_B read from the
// global solution (ancestors are already solved).
template <typename T>
__global__ void k_bwd_init(const FrontD *__restrict__ fr, const T *__restrict__ pool,
                           const int32_t *__restrict__ vars, T *W, const T *__restrict__ Y,
                           const double2 *__restrict__ x, const double *__restrict__ s_in,
                           int64_t sum_m, int64_t n, int nrhs, int f_begin, int max_nrhs) {
    extern __shared__ unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);  // nrhs x kRowsPerCta
    const FrontD f = fr[f_begin + blockIdx.x];
    const int rbase = blockIdx.y * kItemRows;
    if (rbase >= f.p) return;
    const int row = rbase + (threadIdx.x >> 2);
    const bool live = row < f.p;
    const int32_t *v = vars + f.voff;
    T acc[8];
    for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
    for (int c0 = f.p; c0 < f.m; c0 += kRowsPerCta) {
        const int cn = min(kRowsPerCta, f.m - c0);
        __syncthreads();
        for (int idx = threadIdx.x; idx < cn * nrhs; idx += blockDim.x) {
            const int r = idx / cn, cc = idx % cn;
            xs[r * kRowsPerCta + cc] = from_c128<T>(x[r * n + v[c0 + cc]], s_in[r]);
        }
        __syncthreads();
        opener_rows_product(pool + f.f_off, (int64_t)f.ld, row, live, c0, cn, xs, nrhs, acc);
    }
    quad_reduce(acc, nrhs);
    if (live && (threadIdx.x & 3) == 0)
        for (int r = 0; r < nrhs; ++r) W[r * sum_m + f.voff + row] = csub(Y[r * sum_m + f.voff + row], acc[r]);
    (void)max_nrhs;
}

// Backward opener for fronts with a wide boundary, in two deterministic
// passes.  Pass 1: CTA (front, row chunk, column chunk) writes the partial
// product U[rows, cols] x_B[cols] of its 256 x 256 block to scratch; pass 2
// sums the column chunks in a fixed order: acc = y - sum.  Scratch layout
// per front: [col chunk][rhs][row] at bwd_off (elements).
template <typename T>
__global__ void k_bwd_partial(const FrontD *__restrict__ fr, const T *__restrict__ pool,
                              const int32_t *__restrict__ vars, const double2 *__restrict__ x,
                              const int64_t *__restrict__ bwd_off, T *scratch, int64_t n, int nrhs,
                              int f_begin) {
    extern __shared__ unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);  // nrhs x kRowsPerCta
    const int fi = f_begin + blockIdx.x;
    const FrontD f = fr[fi];
    const int rbase = blockIdx.y * kItemRows, c0 = f.p + blockIdx.z * kRowsPerCta;
    if (rbase >= f.p || c0 >= f.m) return;
    const int cn = min(kRowsPerCta, f.m - c0);
    const int32_t *v = vars + f.voff;
    for (int idx = threadIdx.x; idx < cn * nrhs; idx += blockDim.x) {
        const int r = idx / cn, cc = idx % cn;
        xs[r * kRowsPerCta + cc] = from_c128<T>(x[r * n + v[c0 + cc]], 1.0);
    }
    __syncthreads();
    const int row = rbase + (threadIdx.x >> 2);
    const bool live = row < f.p;
    T acc[8];
    for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
    opener_rows_product(pool + f.f_off, (int64_t)f.ld, row, live, c0, cn, xs, nrhs, acc);
    quad_reduce(acc, nrhs);
    if (live && (threadIdx.x & 3) == 0) {
        T *out = scratch + bwd_off[fi] + ((int64_t)blockIdx.z * nrhs) * f.p;
        for (int r = 0; r < nrhs; ++r) out[(int64_t)r * f.p + row] = acc[r];
    }
}

template <typename T>
__global__ void k_bwd_reduce(const FrontD *__restrict__ fr, const int64_t *__restrict__ bwd_off,
                             const T *__restrict__ scratch, T *W, const T *__restrict__ Y, int64_t sum_m,
                             int nrhs, int f_begin) {
    const int fi = f_begin + blockIdx.x;
    const FrontD f = fr[fi];
    const int row = blockIdx.y * kRowsPerCta + threadIdx.x;
    if (row >= f.p) return;
    const int nch = (f.m - f.p + kRowsPerCta - 1) / kRowsPerCta;
    const T *base = scratch + bwd_off[fi];
    for (int r = 0; r < nrhs; ++r) {
        T acc = Y[r * sum_m + f.voff + row];
        for (int c = 0; c < nch; ++c) acc = csub(acc, base[((int64_t)c * nrhs + r) * f.p + row]);
        W[r * sum_m + f.voff + row] = acc;
    }
}

// Backward, one panel (descending k): x_k = inv(U_kk) acc_k, CTA 0 writes
// x_k to the global solution, then acc[0:k0] -= U[0:k0, k] x_k.
template <typename T, typename R>
__global__ void k_bwd_panel(const FrontD *__restrict__ fr, const T *__restrict__ pool,
                            const int32_t *__restrict__ vars, T *W, double2 *x,
                            const double *__restrict__ s_out, int64_t sum_m, int64_t n, int nrhs,
                            int f_begin, int k0) {
    extern __shared__ unsigned char smem_raw[];
    const FrontD f = fr[f_begin + blockIdx.x];
    const int w = min(NB, f.p - k0);
    if (w <= 0) return;
    const int rbase = blockIdx.y * kItemRows;
    if (blockIdx.y > 0 && rbase >= k0) return;
    const T *F = pool + f.f_off;
    const int tid = threadIdx.x;
    T *xk = panel_diag_apply<T, R, true>(F, f.ld, k0, w, W + f.voff, sum_m, nrhs,
                                         reinterpret_cast<T *>(smem_raw));
    if (blockIdx.y == 0) {
        const int32_t *v = vars + f.voff + k0;
        for (int idx = tid; idx < nrhs * w; idx += blockDim.x) {
            const int r = idx / w, row = idx % w;
            x[r * n + v[row]] = to_c128(xk[r * NB + row], s_out[r]);
        }
    }
    panel_rows_update(F, f.ld, k0, w, rbase, k0, xk, nrhs, W + f.voff, sum_m);
}

// Per-column solve scales: s_in = 1/||r||, s_out = sigma ||r||.
__global__ void k_scales(const double *norms, const unsigned long long *maxdiag, int nrhs,
                         double *s_in, double *s_out) {
    const int r = threadIdx.x;
    if (r >= nrhs) return;
    const double nr = norms[r];
    const double sigma = 1.0 / __longlong_as_double((long long)*maxdiag);
    if (nr > 0.0 && isfinite(nr)) {
        s_in[r] = 1.0 / nr;
        s_out[r] = sigma * nr;
    } else {
        s_in[r] = 0.0;
        s_out[r] = 0.0;
    }
}

// P-scaling for transposed solves: P = diag(sxf(i) syf(j)) makes P A
// complex symmetric, so A^T = P A P^-1 and A^-T g = P A^-1 P^-1 g.
// mode 0: out = P^-1 in (multiply by inv_sxf inv_syf); mode 1: out = P in.
__global__ void k_pscale(const double2 *in, double2 *out, const double2 *isxf, const double2 *isyf,
                         int Nx, int Ny, int nrhs, int mode) {
    const int64_t n = (int64_t)Nx * Ny;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n * nrhs;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = k % n;
        const int i = (int)(c / Ny), j = (int)(c % Ny);
        const double2 a = isxf[i], b = isyf[j];
        double2 q = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
        if (mode == 1) {
            const double d = q.x * q.x + q.y * q.y;
            q = make_double2(q.x / d, -q.y / d);
        }
        const double2 v = in[k];
        out[k] = make_double2(v.x * q.x - v.y * q.y, v.x * q.y + v.y * q.x);
    }
}

// ---- GMRES building blocks (FP64, one right-hand side) ----------------------
// Partial dot products h_i = sum conj(V_i) w over a block of the vector for
// i < nv; partial[i * gridDim.x + block].
__global__ void k_multidot_partial(const double2 *__restrict__ V, int64_t n, int nv,
                                   const double2 *__restrict__ w, double2 *partial) {
    __shared__ double2 red[8];
    const int i = blockIdx.y;
    const double2 *vi = V + (size_t)i * n;
    double sr = 0.0, si = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = vi[k], b = w[k];
        sr = fma(a.x, b.x, fma(a.y, b.y, sr));   // conj(a) * b
        si = fma(a.x, b.y, fma(-a.y, b.x, si));
    }
    for (int off = 16; off > 0; off >>= 1) {
        sr += __shfl_down_sync(0xffffffffu, sr, off);
        si += __shfl_down_sync(0xffffffffu, si, off);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(sr, si);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { t.x += red[q].x; t.y += red[q].y; }
        partial[(size_t)i * gridDim.x + blockIdx.x] = t;
    }
    (void)nv;
}
__global__ void k_multidot_final(const double2 *partial, int nparts, double2 *out) {
    __shared__ double2 red[8];
    const int i = blockIdx.x;
    double sr = 0.0, si = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
        sr += partial[(size_t)i * nparts + b].x;
        si += partial[(size_t)i * nparts + b].y;
    }
    for (int off = 16; off > 0; off >>= 1) {
        sr += __shfl_down_sync(0xffffffffu, sr, off);
        si += __shfl_down_sync(0xffffffffu, si, off);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(sr, si);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { t.x += red[q].x; t.y += red[q].y; }
        out[i] = t;
    }
}
// w += sum_i coef_i V_i  (coef on the device, nv <= 32)
__global__ void k_multiaxpy(double2 *w, const double2 *__restrict__ V, int64_t n, int nv,
                           const double2 *__restrict__ coef, double sign) {
    __shared__ double2 c[32];
    if (threadIdx.x < nv) c[threadIdx.x] = coef[threadIdx.x];
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        double2 acc = w[k];
        for (int i = 0; i < nv; ++i) {
            const double2 v = V[(size_t)i * n + k], a = c[i];
            acc.x = fma(sign * a.x, v.x, fma(-sign * a.y, v.y, acc.x));
            acc.y = fma(sign * a.x, v.y, fma(sign * a.y, v.x, acc.y));
        }
        w[k] = acc;
    }
}
__global__ void k_scale_copy(const double2 *__restrict__ in, double2 *out, int64_t n, double s) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = in[k];
        out[k] = make_double2(a.x * s, a.y * s);
    }
}

__global__ void k_axpy(double2 *x, const double2 *d, int64_t len) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < len;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = x[k], b = d[k];
        x[k] = make_double2(a.x + b.x, a.y + b.y);
    }
}

inline int grid1(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

// k_coef over an Nx x Ny operator: column blocks x row runs, the runs sized
// so that the grid is about `ctas` CTAs (one wave) when the grid has rows
// enough.
void coef_launch(const OpDev &o, double2 *coef, int64_t ld, int ctas, cudaStream_t st) {
    const int ncb = (o.Ny + kCoefCols - 1) / kCoefCols;
    const int runs = std::max(1, std::min(o.Nx, ctas / ncb));
    const int rows = (o.Nx + runs - 1) / runs;
    const dim3 grid(ncb, (o.Nx + rows - 1) / rows);
    k_coef<<<grid, kCoefCols, 0, st>>>(o, coef, ld, rows);
}

}  // namespace
}  // namespace fdfd

// ---------------------------------------------------------------------------
// Factor handle.
using namespace fdfd;

struct fdfd_factor {
    fdfd_symbolic *sym = nullptr;
    int precision = FDFD_PREC_C128;
    int max_nrhs = 1;
    int device = 0;
    size_t elem = 16;
    int64_t n = 0;
    // device arrays
    FrontD *d_fronts = nullptr;
    int32_t *d_inv = nullptr;  // per front row: child 0's, then child 1's update-block row (2 x sum_m), or -1
    int32_t *d_piv = nullptr;  // pivot variables front by front (n); level L's are [piv_off[L], piv_off[L + 1])
    std::vector<int64_t> piv_off;
    int32_t *d_vars = nullptr, *d_relmap = nullptr, *d_nbr = nullptr, *d_vfront = nullptr,
            *d_vloc = nullptr;
    void *d_pool = nullptr, *d_W = nullptr, *d_Y = nullptr;
    double2 *d_r = nullptr, *d_d = nullptr, *d_tmp = nullptr;
    double2 *d_isxf = nullptr, *d_isyf = nullptr;
    double *d_partial = nullptr, *d_norm = nullptr, *d_sin = nullptr, *d_sout = nullptr,
           *d_unit = nullptr;
    unsigned long long *d_maxdiag = nullptr;
    int *d_tiny = nullptr;
    double *h_norm = nullptr;  // pinned
    int *h_err = nullptr;      // pinned copy of the solve error flag (and of the tensor-core one)
    // polls of the cooperative solves' bounded waits before they give up
    // (0: the built-in limits; fdfd_factor_set_wait_limit)
    int64_t wait_limit = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // cooperative per-level solves (levels with many panel steps)
    std::vector<char> coop_level;
    int coop_grid = 0;
    int coef_ctas = 152;  // resident k_coef CTAs on the device
    void *d_bar = nullptr;
    int *d_solve_err = nullptr;
    int64_t *d_coop_off = nullptr;
    void *d_coop_scratch = nullptr;
    // pipelined panel units of the cooperative levels (per level: forward
    // list, backward list)
    int2 *d_units = nullptr;
    std::vector<int> unit_fwd_off, unit_fwd_n, unit_bwd_off, unit_bwd_n;
    // two-pass backward opener for levels with wide fronts
    std::vector<char> bwd_wide;
    int64_t *d_bwd_off = nullptr;
    void *d_bwd_scratch = nullptr;
    double pivot_tol = -1.0;  // relative static-pivot threshold (<0: default)
    int fused_max_m = -1;     // largest front factored in one launch (<0: the default of dense_front_fits)
    // coefficients of the factored operator (see k_coef) and the operator
    // description they belong to
    double2 *d_coef = nullptr;
    fdfd_operator coef_op{};
    bool coef_valid = false;
    // look-ahead stream of the tensor-core factorization and its fork/join events
    cudaStream_t st_look = nullptr;
    cudaEvent_t ev_look[2] = {nullptr, nullptr};
    // tensor-core Schur path (FDFD_PREC_C64_TC)
    bool use_tc = false;
    std::vector<char> tc_level;
    // levels whose pivot blocks hold the blocked format (16 x 16 diagonal-
    // block inverses, L and U elsewhere; set by each factorization)
    std::vector<char> blocked_level;
    TcFront *d_tcf = nullptr;
    uint8_t *d_scratch = nullptr;
    int *d_tcerr = nullptr;
    void *d_krylov = nullptr;
    int krylov_m = 0;
    bool numeric_done = false;
    bool has_p = false;  // PML factors known: transposed solves allowed
    int Nx = 0, Ny = 0;
    int batch = 1;   // problems of a batch symbolic (stacked grids, one forest)
    int rows = 0;    // rows per problem
    // the factorization's launch sequence as a CUDA graph (captured at the
    // first factorization, replayed by the later ones: every pointer in it
    // is the factor's own), with the settings it was captured under
    bool use_graphs = true;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t st_cap = nullptr;  // the stream the sequence is captured on
    double graph_pivot_tol = 0.0;
    int graph_fused = 0;
    long long graph_launches[PROF_NCLASS] = {};
    fdfd_factor_stats stats{};
};

namespace fdfd {
namespace {


// A level is factored front-by-front in one launch when all its fronts have
// at most 64 pivots, the largest front fits in shared memory and is at most
// the size limit.  Default: any size for levels of fewer than
// kFusedManyFronts fronts (one launch instead of three per level matters
// for small problems), kWarpMaxM rows for wider levels (larger fronts
// leave one 256-thread CTA an SM and ran faster through the per-panel
// kernels: 2048^2 Hz, 4096 fronts of 155 rows, 54.9 -> 54.2 ms a
// factorization).  Else the caller's limit.
constexpr int kFusedManyFronts = 2048;
template <typename T>
bool dense_front_fits(const fdfd_factor *fac, int maxp, int maxm, int nfl) {
    if (maxp > kDenseMaxPiv || maxm <= 0) return false;
    if (fac->fused_max_m >= 0) {
        if (maxm > fac->fused_max_m) return false;
    } else if (nfl >= kFusedManyFronts && maxm > kWarpMaxM) {
        return false;
    }
    return dense_lu_smem<T>(maxm) <= kDenseSmemMax;
}

// Tensor-core levels with several panels: the diagonal block of panel k+1
// is factored on a second stream while the Schur update of panel k runs.
// Per panel: both triangular updates, the U-panel pack, the update of the
// next panel's 64 columns, then (fork) the next diagonal block on the
// look-ahead stream beside the update of the remaining columns (join
// before the next triangular updates, which need both).
template <typename T, typename R>
int factor_level_lookahead(fdfd_factor *fac, int fb, int nfl, int maxm, int maxp, R tiny, cudaStream_t st) {
    T *pool = (T *)fac->d_pool;
    cudaStream_t s2 = fac->st_look;
    constexpr int kNextTiles = NB / kTileNc;  // column tiles of the next panel
    prof_begin(PROF_LU_DIAG, st);
    dense_lu_launch<T, R>(nfl, NB, st, fac->d_fronts, pool, fb, 0, 0, 0, tiny, fac->d_tiny);
    prof_end(PROF_LU_DIAG, st, 1);
    for (int k0 = 0; k0 < maxp; k0 += NB) {
        const int trail = maxm - k0 - 1;  // upper bound of m - t0
        if (trail <= 0) continue;
        prof_begin(PROF_TRSM, st);
        trsm_launch<T, R>(nfl, trail, std::min(NB, maxp - k0), st, fac->d_fronts, pool, fb, k0, fac->d_tcf,
                          fac->d_scratch);
        prof_end(PROF_TRSM, st, 1);
        prof_begin(PROF_SCHUR, st);
        int rc = FDFD_OK;
        const bool next = k0 + NB < maxp;
        if (next) {
            rc = tc_schur_cols(fac->d_tcf, (c64 *)pool, fb, nfl, k0, trail, 0, kNextTiles, fac->d_scratch,
                               fac->d_tcerr, st);
            if (rc) return rc;
            CUDA_TRY(cudaEventRecord(fac->ev_look[0], st));
            CUDA_TRY(cudaStreamWaitEvent(s2, fac->ev_look[0], 0));
            prof_begin(PROF_LU_DIAG, s2);
            dense_lu_launch<T, R>(nfl, NB, s2, fac->d_fronts, pool, fb, k0 + NB, 0, 0, tiny, fac->d_tiny);
            prof_end(PROF_LU_DIAG, s2, 1);
            CUDA_TRY(cudaEventRecord(fac->ev_look[1], s2));
        }
        rc = tc_schur_cols(fac->d_tcf, (c64 *)pool, fb, nfl, k0, trail, next ? kNextTiles : 0, 1 << 30,
                           fac->d_scratch, fac->d_tcerr, st);
        if (rc) return rc;
        prof_end(PROF_SCHUR, st, next ? 2 : 1);
        if (next) CUDA_TRY(cudaStreamWaitEvent(st, fac->ev_look[1], 0));
    }
    return FDFD_OK;
}

template <typename T, typename R>
int factor_levels(fdfd_factor *fac, const OpDev &o, cudaStream_t st) {
    const Symbolic &S = fac->sym->s;
    // Every front above the leaves is written whole by the parent-side
    // extend-add and then takes its operator entries; the leaves (level 0),
    // when factored whole, assemble their fronts in the LU kernel, else
    // their part of the pool is cleared and assembled here.  No other part
    // of the pool is cleared.
    const bool leaf_asm = dense_front_fits<T>(fac, S.lev_max_p[0], S.lev_max_m[0], S.level_ptr[1] - S.level_ptr[0]);
    const int64_t leaf_entries = S.nlev > 1 ? S.pool_off[S.level_ptr[1]] : S.pool_entries;
    if (!leaf_asm) CUDA_TRY(cudaMemsetAsync(fac->d_pool, 0, (size_t)leaf_entries * sizeof(T), st));
    CUDA_TRY(cudaMemsetAsync(fac->d_tiny, 0, sizeof(int), st));
    if (fac->d_tcerr) CUDA_TRY(cudaMemsetAsync(fac->d_tcerr, 0, sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(fac->d_maxdiag, 0, sizeof(unsigned long long), st));
    prof_begin(PROF_ASSEMBLE, st);
    k_maxdiag<<<std::min(grid1(fac->n), 152 * 4), 256, 0, st>>>(o, fac->d_maxdiag);  // many entries a thread
    if (!leaf_asm)
        k_assemble_fronts<T><<<grid1(fac->n), 256, 0, st>>>(o, fac->d_fronts, fac->d_vfront, fac->d_vloc, fac->d_nbr,
                                                           fac->d_maxdiag, (T *)fac->d_pool, 0, S.level_ptr[1]);
    prof_end(PROF_ASSEMBLE, st, leaf_asm ? 1 : 2);
    // Default static-pivot thresholds (relative to max|diag A|): sqrt(eps)
    // for complex128; 1e-5 for complex64, the value that minimised the
    // refinement steps of the 2048^2 Hz workload (sqrt(eps_f32) = 3.4e-4
    // lifted 22 pivots and needed 10 steps, 1e-5 lifted 2 and needed 6,
    // smaller thresholds lifted none and needed 10).
    const double def = std::is_same<R, float>::value ? 1e-5 : std::sqrt((double)std::numeric_limits<R>::epsilon());
    const R tiny = (R)(fac->pivot_tol >= 0.0 ? fac->pivot_tol : def);
    T *pool = (T *)fac->d_pool;
    fac->blocked_level.assign(S.nlev, 0);
    for (int L = 0; L < S.nlev; ++L) {
        const int fb = S.level_ptr[L], nfl = S.level_ptr[L + 1] - fb;
        if (L > 0) {
            // about 2048 entries per CTA; at most (1 << 30) / maxm columns so idx fits in int
            const int maxm_l = S.lev_max_m[L];
            const int cb = std::max(1, 2048 / maxm_l);
            dim3 g(nfl, (maxm_l + cb - 1) / cb);
            prof_begin(PROF_EXTEND_ADD, st);
            k_extend_pull<T><<<g, 256, 0, st>>>(fac->d_fronts, fac->d_inv, fac->d_inv + S.sum_m, pool, fb, cb);
            prof_end(PROF_EXTEND_ADD, st, 1);
            prof_begin(PROF_ASSEMBLE, st);
            const int np = (int)(fac->piv_off[L + 1] - fac->piv_off[L]);
            k_assemble_level<T><<<std::max(1, (np + 255) / 256), 256, 0, st>>>(
                o, fac->d_fronts, fac->d_piv + fac->piv_off[L], np, fac->d_vfront, fac->d_vloc, fac->d_nbr,
                fac->d_maxdiag, pool);
            prof_end(PROF_ASSEMBLE, st, 1);
        }
        const int maxm = S.lev_max_m[L], maxp = S.lev_max_p[L];
        if (dense_front_fits<T>(fac, maxp, maxm, nfl)) {
            // every front of the level in one launch: LU, L21, U12 and the update matrix
            prof_begin(PROF_LU_DIAG, st);
            // levels solved one warp per front keep the blocked pivot-block format
            const int blocked = maxm <= kWarpMaxM ? 1 : 0;
            fac->blocked_level[L] = (char)blocked;
            LeafAsm la;
            if (L == 0 && leaf_asm) {
                la.o = o;
                la.vars = fac->d_vars;
                la.nbr_loc = fac->d_nbr;
                la.maxdiag = fac->d_maxdiag;
            }
            dense_lu_launch<T, R>(nfl, (maxm + 15) / 16 * 16, st, fac->d_fronts, pool, fb, 0, 1, blocked, tiny,
                                  fac->d_tiny, la);
            prof_end(PROF_LU_DIAG, st, 1);
            continue;
        }
        const bool tc = std::is_same<T, c64>::value && fac->use_tc && fac->tc_level[L];
        if (tc && maxp > NB && fac->st_look) {
            int rc = factor_level_lookahead<T, R>(fac, fb, nfl, maxm, maxp, tiny, st);
            if (rc) return rc;
            continue;
        }
        for (int k0 = 0; k0 < maxp; k0 += NB) {
            prof_begin(PROF_LU_DIAG, st);
            dense_lu_launch<T, R>(nfl, NB, st, fac->d_fronts, pool, fb, k0, 0, 0, tiny, fac->d_tiny);
            prof_end(PROF_LU_DIAG, st, 1);
            const int trail = maxm - k0 - 1;  // upper bound of m - t0
            if (trail <= 0) continue;
            const int tiles = (trail + BM - 1) / BM;
            prof_begin(PROF_TRSM, st);
            trsm_launch<T, R>(nfl, trail, std::min(NB, maxp - k0), st, fac->d_fronts, pool, fb, k0,
                              tc ? fac->d_tcf : nullptr, tc ? fac->d_scratch : nullptr);
            prof_end(PROF_TRSM, st, 1);
            if (tc) {
                prof_begin(PROF_SCHUR, st);
                int rc = tc_schur_cols(fac->d_tcf, (c64 *)fac->d_pool, fb, nfl, k0, trail, 0, 1 << 30, fac->d_scratch,
                                   fac->d_tcerr, st);
                if (rc) return rc;
                prof_end(PROF_SCHUR, st, 1);
            } else {
                prof_begin(PROF_SCHUR_SIMT, st);
                k_schur_simt<T, R><<<dim3(nfl, tiles, tiles), 256, 0, st>>>(fac->d_fronts, pool, fb, k0);
                prof_end(PROF_SCHUR_SIMT, st, 1);
            }
        }
    }
    CUDA_TRY(cudaGetLastError());
    return FDFD_OK;
}

// The factorization from the coefficient store through the last level as a
// CUDA graph.  Everything the sequence touches belongs to the factor (pool,
// index lists, coefficient store, scratch, the look-ahead stream's events),
// so the graph captured at the first call is replayed by every later one;
// only the coefficient evaluation (k_coef, which reads the caller's
// operator buffers) runs outside it.  The capture runs on a stream of the
// factor's own (capturing records launches without running them, and the
// caller's stream may be the legacy default stream, which cannot be
// captured); the graph is then launched on the caller's stream.  A graph is
// not used while per-class profiling is on (replays are not timed per
// class), for an explicit-stencil operator read in place, while the
// caller's stream is itself being captured (its graph takes the launches),
// or once a capture has failed.
template <typename T, typename R>
int factor_levels_graphed(fdfd_factor *fac, const OpDev &o, cudaStream_t st) {
    if (!fac->use_graphs || prof_enabled() || o.stencil != fac->d_coef) return factor_levels<T, R>(fac, o, st);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return factor_levels<T, R>(fac, o, st);
    }
    if (fac->graph && fac->graph_pivot_tol == fac->pivot_tol && fac->graph_fused == fac->fused_max_m) {
        CUDA_TRY(cudaGraphLaunch(fac->graph, st));
        for (int c = 0; c < PROF_NCLASS; ++c) prof_count(c, fac->graph_launches[c]);
        return FDFD_OK;
    }
    if (fac->graph) {
        cudaGraphExecDestroy(fac->graph);
        fac->graph = nullptr;
    }
    // the captured sequence sees only the scalars and the factor's own store
    OpDev og{};
    og.Nx = o.Nx;
    og.Ny = o.Ny;
    og.Nxp = o.Nxp;
    og.pol = o.pol;
    og.stencil = fac->d_coef;
    long long before[PROF_NCLASS];
    for (int c = 0; c < PROF_NCLASS; ++c) before[c] = prof_launches(c);
    if ((!fac->st_cap && cudaStreamCreateWithFlags(&fac->st_cap, cudaStreamNonBlocking) != cudaSuccess) ||
        cudaStreamBeginCapture(fac->st_cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        fac->use_graphs = false;
        return factor_levels<T, R>(fac, o, st);
    }
    const int rc = factor_levels<T, R>(fac, og, fac->st_cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(fac->st_cap, &g);
    if (rc == FDFD_OK && e == cudaSuccess) e = cudaGraphInstantiate(&fac->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (rc != FDFD_OK || e != cudaSuccess) {
        // not capturable here: launch directly from now on (the launch
        // counts of the failed capture are taken back)
        cudaGetLastError();
        for (int c = 0; c < PROF_NCLASS; ++c) prof_count(c, before[c] - prof_launches(c));
        fac->graph = nullptr;
        fac->use_graphs = false;
        return factor_levels<T, R>(fac, o, st);
    }
    for (int c = 0; c < PROF_NCLASS; ++c) fac->graph_launches[c] = prof_launches(c) - before[c];
    fac->graph_pivot_tol = fac->pivot_tol;
    fac->graph_fused = fac->fused_max_m;
    CUDA_TRY(cudaGraphLaunch(fac->graph, st));
    return FDFD_OK;
}

// ---- cooperative per-level solves --------------------------------------------
// Levels with many panel steps (the few large fronts near the root) run each
// direction of the substitution as ONE cooperative launch: the grid walks
// the panel steps itself, separated by a grid-wide barrier, instead of one
// launch per step.  The barrier's wait is bounded: after kBarLimit polls a
// CTA records an error and returns (the solve is then reported as failed).
struct GridBar {
    unsigned int count, gen;
};
constexpr unsigned kBarLimit = 1u << 24;

// `limit`: polls before giving up (kBarLimit by default; a factor's wait
// limit, fdfd_factor_set_wait_limit, replaces it).
__device__ bool grid_sync(GridBar *gb, int *err, unsigned limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &gb->gen;
        const unsigned int g = *vgen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&gb->count, 1u) == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            for (unsigned int it = 0; *vgen == g; ++it) {
                if (it >= limit) {
                    ok = 0;
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Values passed between the pipelined panel units of one launch carry their
// own readiness.  Before the launch's grid barrier every slot a unit will
// publish into is set to kUnset, a signalling-NaN bit pattern that no
// arithmetic produces (NaN results are quiet), in each 32-bit half of a
// complex64 slot and each 64-bit half of a complex128 slot.  The producing
// unit stores the value with relaxed gpu-scope stores; a consumer polls each
// slot with relaxed gpu-scope loads until no half carries the pattern, so no
// separate flag, fence or second read is on the chain between units.  The
// poll is bounded: after kFlagLimit rounds, or once another CTA has reported
// a failure, the CTA records the error and the block returns.
constexpr unsigned kFlagLimit = 1u << 22;
constexpr unsigned kUnset32 = 0x7fa5a5a5u;

// The limits a factor's cooperative solves use (its wait limit, if set).
unsigned bar_limit_of(const fdfd_factor *fac) {
    return fac->wait_limit > 0 ? (unsigned)std::min<int64_t>(fac->wait_limit, kBarLimit) : kBarLimit;
}
unsigned flag_limit_of(const fdfd_factor *fac) {
    return fac->wait_limit > 0 ? (unsigned)std::min<int64_t>(fac->wait_limit, kFlagLimit) : kFlagLimit;
}
constexpr unsigned long long kUnset64 = 0x7ff4a5a5a5a5a5a5ull;

__device__ __forceinline__ void set_unset(c64 *p) {
    *reinterpret_cast<uint2 *>(p) = make_uint2(kUnset32, kUnset32);
}
__device__ __forceinline__ void set_unset(c128 *p) {
    *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(kUnset64, kUnset64);
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const void *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(void *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void put_value(c64 *p, c64 v) {
    st_relaxed_u64(p, (unsigned long long)__float_as_uint(v.x) |
                          ((unsigned long long)__float_as_uint(v.y) << 32));
}
__device__ __forceinline__ void put_value(c128 *p, c128 v) {
    st_relaxed_u64(p, (unsigned long long)__double_as_longlong(v.x));
    st_relaxed_u64(reinterpret_cast<double *>(p) + 1, (unsigned long long)__double_as_longlong(v.y));
}

__device__ __forceinline__ bool try_take(const c64 *p, c64 &out) {
    const unsigned long long v = ld_relaxed_u64(p);
    const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
    if (lo == kUnset32 || hi == kUnset32) return false;
    out = cmake<float>(__uint_as_float(lo), __uint_as_float(hi));
    return true;
}
__device__ __forceinline__ bool try_take(const c128 *p, c128 &out) {
    const unsigned long long re = ld_relaxed_u64(p);
    const unsigned long long im = ld_relaxed_u64(reinterpret_cast<const double *>(p) + 1);
    if (re == kUnset64 || im == kUnset64) return false;
    out = cmake<double>(__longlong_as_double((long long)re), __longlong_as_double((long long)im));
    return true;
}

// Stage one published panel (nrhs x w values at vsrc[r * sum_m + c0 + i])
// into vs (nrhs x NB, zero past w), waiting for each value.
template <typename T>
__device__ bool take_panel(const T *vsrc, int64_t sum_m, int c0, int w, int nrhs, T *vs, int *err,
                           unsigned limit) {
    int fail = 0;
    for (int idx = threadIdx.x; idx < nrhs * NB && !fail; idx += blockDim.x) {
        const int r = idx / NB, i = idx % NB;
        T v = czero<T>();
        if (i < w) {
            const T *src = vsrc + r * sum_m + c0 + i;
            for (unsigned it = 0; !try_take(src, v); ++it) {
                if (it >= limit || ((it & 1023u) == 1023u && *(volatile int *)err != 0)) {
                    fail = 1;
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(16);
            }
        }
        vs[idx] = v;
    }
    return __syncthreads_or(fail) == 0;
}

template <typename T>
__device__ __forceinline__ T ldcg_c(const T *p);
template <>
__device__ __forceinline__ c64 ldcg_c<c64>(const c64 *p) {
    const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return cmake<float>(v.x, v.y);
}
template <>
__device__ __forceinline__ c128 ldcg_c<c128>(const c128 *p) {
    const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
    return cmake<double>(v.x, v.y);
}

// Pipelined panel unit, the shared part: acc[rhs] (four partial sums per
// row, rows rr = tid / 4 of the block) -= F[rows, panel] v_panel for each
// panel in order, where v_panel (a 64-vector per rhs) is taken from vsrc
// (stride sum_m) as its values are published.  The panel's matrix tile is
// loaded before the wait.
template <typename T, int N>
__device__ __forceinline__ bool unit_panels(const T *F, int64_t ld, int r0, bool live, int k_first, int k_last,
                                            int k_step, int p, const T *vsrc, int64_t sum_m, int nrhs, int *err,
                                            unsigned flag_limit, T *vs, T (&acc)[N]) {
    const int rr = threadIdx.x >> 2, t0 = 16 * (threadIdx.x & 3);
    // the tile of the next panel is loaded while this panel waits and computes
    T a[16], an[16];
    if (k_first != k_last) {
        const int w = min(NB, p - k_first * NB);
#pragma unroll
        for (int i = 0; i < 16; ++i)
            an[i] = (live && t0 + i < w) ? F[(r0 + rr) + (int64_t)(k_first * NB + t0 + i) * ld] : czero<T>();
    }
    for (int k = k_first; k != k_last; k += k_step) {
        const int c0 = k * NB, w = min(NB, p - c0);
#pragma unroll
        for (int i = 0; i < 16; ++i) a[i] = an[i];
        if (k + k_step != k_last) {
            const int cn = (k + k_step) * NB, wn = min(NB, p - cn);
#pragma unroll
            for (int i = 0; i < 16; ++i)
                an[i] = (live && t0 + i < wn) ? F[(r0 + rr) + (int64_t)(cn + t0 + i) * ld] : czero<T>();
        }
        if (!take_panel(vsrc, sum_m, c0, w, nrhs, vs, err, flag_limit)) return false;
        for (int r = 0; r < nrhs; ++r) {
            const T *vr = vs + r * NB + t0;
#pragma unroll
            for (int i = 0; i < 16; ++i) cmac(acc[r], a[i], vr[i]);
        }
        __syncthreads();
    }
    return true;
}

// Stage the triangle of the diagonal block's inverse (UPPER: on and above
// the diagonal; else strictly below) into Ds (ld NB).
template <typename T, bool UPPER>
__device__ __forceinline__ void stage_diag(const T *F, int64_t ld, int r0, int rn, T *Ds) {
    for (int c = threadIdx.x >> 6; c < rn; c += blockDim.x >> 6) {
        const int r = threadIdx.x & 63;
        if (r < rn) {
            const bool need = UPPER ? (r <= c) : (r > c);
            Ds[r + c * NB] = need ? F[(r0 + r) + (int64_t)(r0 + c) * ld] : czero<T>();
        }
    }
}

// out[rhs][row] = sum_t Ds[row, t] vin[rhs][t] (+ vin[row] for the unit lower
// inverse), four threads per row; returns the value for q == 0 threads.
template <typename T, bool UPPER>
__device__ __forceinline__ T diag_rows(const T *Ds, const T *vr, int rn, int row) {
    const int q = threadIdx.x & 3;
    T s = czero<T>();
    if (row < rn) {
        if (UPPER) {
            for (int t = row + q; t < rn; t += 4) cmac(s, Ds[row + t * NB], vr[t]);
        } else {
            for (int t = q; t < row; t += 4) cmac(s, Ds[row + t * NB], vr[t]);
        }
    }
    for (int off = 1; off < 4; off <<= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, off);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, off);
    }
    if (!UPPER && row < rn) s = cadd(s, vr[row]);
    return s;
}

template <typename T, typename R, int NR>
__global__ void __launch_bounds__(kRowsPerCta, sizeof(T) == 8 ? 3 : 1)
    k_fwd_level(const FrontD *__restrict__ fr, int fb, int nfl, int maxp, int maxm, const T *__restrict__ pool,
                const int32_t *__restrict__ vars, const int32_t *__restrict__ inv0, const int32_t *__restrict__ inv1,
                const double2 *__restrict__ b, const double *__restrict__ s_in, T *W, T *Y, int64_t sum_m,
                int64_t n, int nrhs, GridBar *gb, int *err, const int2 *__restrict__ units, int nunits,
                unsigned bar_limit, unsigned flag_limit) {
    if (NR == 1) nrhs = 1;  // one right-hand side: the sums stay in registers
    extern __shared__ unsigned char smem_raw[];
    const int tid = threadIdx.x;
    // gather, spread over every CTA (one entry a thread): w = s_in b on the
    // pivots (zero on the boundary), plus child 0's update, plus child 1's
    // -- the inverse maps give each parent row its children's update rows --
    // added in that order; the pivot slots of Y are marked unpublished
    const int gchunks = (maxm + (int)blockDim.x - 1) / (int)blockDim.x;
    for (int item = blockIdx.x; item < nfl * gchunks; item += gridDim.x) {
        const int fi = item / gchunks, k = (item - fi * gchunks) * (int)blockDim.x + tid;
        const FrontD f = fr[fb + fi];
        if (k >= f.m) continue;
        const int a0 = f.c0 >= 0 ? inv0[f.voff + k] : -1, a1 = f.c1 >= 0 ? inv1[f.voff + k] : -1;
        const int64_t o0 = a0 >= 0 ? (int64_t)fr[f.c0].voff + fr[f.c0].p + a0 : 0;
        const int64_t o1 = a1 >= 0 ? (int64_t)fr[f.c1].voff + fr[f.c1].p + a1 : 0;
        const int var = k < f.p ? vars[f.voff + k] : 0;
        for (int r = 0; r < nrhs; ++r) {
            T v = (k < f.p) ? from_c128<T>(b[r * n + var], s_in[r]) : czero<T>();
            if (a0 >= 0) v = cadd(v, W[r * sum_m + o0]);
            if (a1 >= 0) v = cadd(v, W[r * sum_m + o1]);
            W[r * sum_m + f.voff + k] = v;
            if (k < f.p) set_unset(Y + r * sum_m + f.voff + k);
        }
    }
    if (!grid_sync(gb, err, bar_limit)) return;
    (void)maxp;
    // pipelined panels: unit (front, row block R); a pivot block computes
    // y_R = inv(L_RR) (w_R - sum_k L[R, k] y_k) and publishes it, an update
    // block accumulates w_B -= sum_k L[B, k] y_k for the parent's gather
    T *sm = reinterpret_cast<T *>(smem_raw);
    T *Ds = sm, *vin = sm + NB * NB;
    const int rr = tid >> 2, q = tid & 3;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int2 un = units[u];
        const int fi = un.x, rb = un.y;
        const FrontD f = fr[fb + fi];
        const int KP = (f.p + NB - 1) / NB;
        const bool piv = rb < KP;
        const int r0 = piv ? rb * NB : f.p + (rb - KP) * NB;
        const int rn = min(NB, (piv ? f.p : f.m) - r0);
        const T *F = pool + f.f_off;
        const int64_t ld = f.ld;
        const bool live = rr < rn;
        // the pivot rows of w are final since the gather: load them now, off
        // the chain between units (each row's q == 0 thread reads back its own)
        T *wpre = vin + nrhs * NB;
        if (piv && live && q == 0)
            for (int r = 0; r < nrhs; ++r) wpre[r * NB + rr] = ldcg_c(W + r * sum_m + f.voff + r0 + rr);
        if (piv) stage_diag<T, false>(F, ld, r0, rn, Ds);
        T acc[NR];
        for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
        if (!unit_panels(F, ld, r0, live, 0, piv ? rb : KP, 1, f.p, Y + f.voff, sum_m, nrhs, err, flag_limit, vin,
                         acc))
            return;
        quad_reduce(acc, nrhs);
        if (piv) {
            if (live && q == 0)
                for (int r = 0; r < nrhs; ++r) vin[r * NB + rr] = csub(wpre[r * NB + rr], acc[r]);
            __syncthreads();
            for (int r = 0; r < nrhs; ++r) {
                const T y = diag_rows<T, false>(Ds, vin + r * NB, rn, rr);
                if (live && q == 0) put_value(Y + r * sum_m + f.voff + r0 + rr, y);
            }
        } else if (live && q == 0) {
            for (int r = 0; r < nrhs; ++r) {
                T *d = W + r * sum_m + f.voff + r0 + rr;
                *d = csub(ldcg_c(d), acc[r]);
            }
        }
        __syncthreads();
    }
}

template <typename T, typename R, int NR>
__global__ void __launch_bounds__(kRowsPerCta, sizeof(T) == 8 ? 3 : 1)
    k_bwd_level(const FrontD *__restrict__ fr, int fb, int nfl, int maxp, int maxb, const T *__restrict__ pool,
                const int32_t *__restrict__ vars, double2 *x, const int64_t *__restrict__ bwd_off, T *scratch,
                T *W, T *Y, int64_t sum_m, int64_t n, int nrhs, GridBar *gb, int *err,
                const int2 *__restrict__ units, int nunits, unsigned bar_limit, unsigned flag_limit) {
    if (NR == 1) nrhs = 1;  // one right-hand side: the sums stay in registers
    extern __shared__ unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);  // opener: nrhs x kRowsPerCta; panels: panel layout
    const int tid = threadIdx.x;
    const int prow = (maxp + kItemRows - 1) / kItemRows;
    const int cch = max(1, (maxb + kRowsPerCta - 1) / kRowsPerCta);
    // opener, pass 1: partial products U[rows, cols] x_B[cols] per 64 x 256 block
    for (int item = blockIdx.x; item < nfl * prow * cch; item += gridDim.x) {
        const int fi = item / (prow * cch), rc = (item / cch) % prow, cc = item % cch;
        const FrontD f = fr[fb + fi];
        const int rbase = rc * kItemRows, c0 = f.p + cc * kRowsPerCta;
        if (rbase >= f.p || c0 >= f.m) continue;
        const int cn = min(kRowsPerCta, f.m - c0);
        const int32_t *v = vars + f.voff;
        for (int idx = tid; idx < cn * nrhs; idx += blockDim.x) {
            const int r = idx / cn, q = idx % cn;
            xs[r * kRowsPerCta + q] = from_c128<T>(x[r * n + v[c0 + q]], 1.0);
        }
        __syncthreads();
        const int row = rbase + (tid >> 2);
        const bool live = row < f.p;
        T acc[NR];
        for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
        opener_rows_product(pool + f.f_off, (int64_t)f.ld, row, live, c0, cn, xs, nrhs, acc);
        quad_reduce(acc, nrhs);
        if (live && (tid & 3) == 0) {
            T *out = scratch + bwd_off[fb + fi] + ((int64_t)cc * nrhs) * f.p;
            for (int r = 0; r < nrhs; ++r) out[(int64_t)r * f.p + row] = acc[r];
        }
        __syncthreads();
    }
    // the pivot slots of W (free in the backward pass) become the
    // publication slots of x: marked unpublished before the grid barrier
    const int prow2 = (maxp + kRowsPerCta - 1) / kRowsPerCta;
    for (int item = blockIdx.x; item < nfl * prow2; item += gridDim.x) {
        const int fi = item / prow2, row = (item % prow2) * kRowsPerCta + tid;
        const FrontD f = fr[fb + fi];
        if (row < f.p)
            for (int r = 0; r < nrhs; ++r) set_unset(W + r * sum_m + f.voff + row);
    }
    if (!grid_sync(gb, err, bar_limit)) return;
    // pipelined panels, descending: x_R = inv(U_RR) (acc_R - sum_{j>R} U[R, j] x_j),
    // with acc = y - the opener's column blocks (summed in a fixed order);
    // x published in W's pivot rows (and written to the global solution)
    T *Ds = xs, *vin = xs + NB * NB;
    const int rr = tid >> 2, q = tid & 3;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int2 un = units[u];
        const int fi = un.x, rb = un.y;
        const FrontD f = fr[fb + fi];
        const int KP = (f.p + NB - 1) / NB;
        const int r0 = rb * NB, rn = min(NB, f.p - r0);
        const T *F = pool + f.f_off;
        const int64_t ld = f.ld;
        const bool live = rr < rn;
        // this unit's rows of acc, final since the opener: formed off the
        // chain between units
        T *wpre = vin + nrhs * NB;
        if (live && q == 0) {
            const int nch = (f.m - f.p + kRowsPerCta - 1) / kRowsPerCta;
            const T *base = scratch + bwd_off[fb + fi];
            for (int r = 0; r < nrhs; ++r) {
                T a = Y[r * sum_m + f.voff + r0 + rr];
                for (int c = 0; c < nch; ++c) a = csub(a, base[((int64_t)c * nrhs + r) * f.p + r0 + rr]);
                wpre[r * NB + rr] = a;
            }
        }
        stage_diag<T, true>(F, ld, r0, rn, Ds);
        T acc[NR];
        for (int r = 0; r < nrhs; ++r) acc[r] = czero<T>();
        if (!unit_panels(F, ld, r0, live, KP - 1, rb, -1, f.p, W + f.voff, sum_m, nrhs, err, flag_limit, vin,
                         acc))
            return;
        quad_reduce(acc, nrhs);
        if (live && q == 0)
            for (int r = 0; r < nrhs; ++r) vin[r * NB + rr] = csub(wpre[r * NB + rr], acc[r]);
        __syncthreads();
        const int32_t *v = vars + f.voff + r0;
        for (int r = 0; r < nrhs; ++r) {
            const T xv = diag_rows<T, true>(Ds, vin + r * NB, rn, rr);
            if (live && q == 0) {
                put_value(W + r * sum_m + f.voff + r0 + rr, xv);
                x[r * n + v[rr]] = to_c128(xv, 1.0);
            }
        }
        __syncthreads();
    }
}

template <typename T, typename R>
int set_smem_attrs() {
    CUDA_TRY(cudaFuncSetAttribute(k_dense_lu<T, R, 0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDenseSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_dense_lu<T, R, 64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDenseSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_dense_lu<T, R, 80, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDenseSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_dense_lu<T, R, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDenseSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_dense_lu<T, R, 80, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDenseSmemMax));

    const int ps = (int)std::max(panel_smem_bytes<T>(8), (size_t)8 * kRowsPerCta * sizeof(T));
    CUDA_TRY(cudaFuncSetAttribute(k_fwd_panel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_bwd_panel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_fwd_level<T, R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_fwd_level<T, R, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_bwd_level<T, R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_bwd_level<T, R, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps));
    CUDA_TRY(cudaFuncSetAttribute(k_fwd_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_fwd_warp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_bwd_warp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmemMax));
    CUDA_TRY(cudaFuncSetAttribute(k_bwd_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmemMax));
    return FDFD_OK;
}

// x = A^-1 b for nrhs columns (b, x complex128 on device; may alias d_tmp).
// s_in / s_out are device arrays of per-column scales.
// Levels whose fronts all have at most 64 pivots take the one-launch steps
// of each direction when their vectors fit in shared memory.
template <typename T>
bool warp_level_fits(int maxp, int maxm, int nrhs) {
    return maxp <= NB && maxm <= kWarpMaxM && warp_smem_bytes<T>(nrhs, maxm) <= kSmallSmemMax;
}
template <typename T>
bool small_level_fits(int maxp, int maxm, int nrhs) {
    return maxp <= NB && maxm <= kSmallMaxM && small_smem_bytes<T>(nrhs, maxm) <= kSmallSmemMax;
}

template <typename T, typename R>
int solve_levels(fdfd_factor *fac, const double2 *b, const double *s_in, double2 *x, int nrhs, cudaStream_t st) {
    const Symbolic &S = fac->sym->s;
    T *W = (T *)fac->d_W, *Y = (T *)fac->d_Y;
    const T *pool = (const T *)fac->d_pool;
    const int64_t sum_m = S.sum_m, n = fac->n;
    const size_t sm_panel = panel_smem_bytes<T>(nrhs);
    CUDA_TRY(cudaMemsetAsync(fac->d_bar, 0, sizeof(GridBar), st));
    const size_t sm_coop = std::max(panel_smem_bytes<T>(nrhs), (size_t)nrhs * kRowsPerCta * sizeof(T));
    for (int L = 0; L < S.nlev; ++L) {
        const int fb = S.level_ptr[L], nfl = S.level_ptr[L + 1] - fb;
        prof_begin(PROF_SOLVE_FWD, st);
        if (fac->coop_level[L]) {
            int maxp = S.lev_max_p[L], maxm = S.lev_max_m[L];
            GridBar *gb = (GridBar *)fac->d_bar;
            int *err = fac->d_solve_err;
            const int2 *units = fac->d_units + fac->unit_fwd_off[L];
            int nunits = fac->unit_fwd_n[L];
            unsigned bar_limit = bar_limit_of(fac), flag_limit = flag_limit_of(fac);
            const int32_t *inv0 = fac->d_inv, *inv1 = fac->d_inv + S.sum_m;
            void *args[] = {(void *)&fac->d_fronts, (void *)&fb, (void *)&nfl, (void *)&maxp, (void *)&maxm,
                            (void *)&pool, (void *)&fac->d_vars, (void *)&inv0, (void *)&inv1, (void *)&b,
                            (void *)&s_in, (void *)&W, (void *)&Y, (void *)&sum_m, (void *)&n, (void *)&nrhs,
                            (void *)&gb, (void *)&err,
                            (void *)&units, (void *)&nunits, (void *)&bar_limit, (void *)&flag_limit};
            // grid: the most work items any phase of this level has, capped
            // at the co-resident limit
            const int items = std::max(nfl, nunits);
            const int grid = std::max(1, std::min(fac->coop_grid, items));
            CUDA_TRY(cudaLaunchCooperativeKernel(nrhs == 1 ? (const void *)k_fwd_level<T, R, 1> : (const void *)k_fwd_level<T, R, 8>, dim3(grid),
                                                 dim3(kRowsPerCta), args, sm_coop, st));
            prof_end(PROF_SOLVE_FWD, st, 1);
            continue;
        }
        const int maxm = S.lev_max_m[L], maxp = S.lev_max_p[L];
        if (warp_level_fits<T>(maxp, maxm, nrhs)) {
            k_fwd_warp<T><<<(nfl + kWarpFronts - 1) / kWarpFronts, 32 * kWarpFronts, warp_smem_bytes<T>(nrhs, maxm),
                            st>>>(fac->d_fronts, fac->d_vars, fac->d_inv, fac->d_inv + S.sum_m, pool, b, s_in, W, Y,
                                  sum_m, n, nrhs, fb, nfl, maxm, (int)fac->blocked_level[L]);
            prof_end(PROF_SOLVE_FWD, st, 1);
            continue;
        }
        if (small_level_fits<T>(maxp, maxm, nrhs)) {
            k_fwd_small<T><<<nfl, kSmallThreads, small_smem_bytes<T>(nrhs, maxm), st>>>(
                fac->d_fronts, fac->d_vars, fac->d_inv, fac->d_inv + S.sum_m, pool, b, s_in, W, Y, sum_m, n, nrhs,
                fb, maxm);
            prof_end(PROF_SOLVE_FWD, st, 1);
            continue;
        }
        k_fwd_gather<T><<<nfl, 256, 0, st>>>(fac->d_fronts, fac->d_vars, fac->d_relmap, b, s_in, W, sum_m, n,
                                             nrhs, fb);
        int nl = 1;
        for (int k0 = 0; k0 < maxp; k0 += NB, ++nl) {
            const int rows = std::max(1, (maxm - k0 + kItemRows - 1) / kItemRows);
            k_fwd_panel<T, R><<<dim3(nfl, rows), kRowsPerCta, sm_panel, st>>>(fac->d_fronts, pool, W, Y,
                                                                            sum_m, nrhs, fb, k0);
        }
        prof_end(PROF_SOLVE_FWD, st, nl);
    }
    for (int L = S.nlev - 1; L >= 0; --L) {
        const int fb = S.level_ptr[L], nfl = S.level_ptr[L + 1] - fb;
        const int maxp = S.lev_max_p[L];
        const int prow = (maxp + kItemRows - 1) / kItemRows;
        prof_begin(PROF_SOLVE_BWD, st);
        if (fac->coop_level[L]) {
            int maxpp = maxp, maxb = 0;
            for (int f = fb; f < fb + nfl; ++f) maxb = std::max(maxb, S.m[f] - S.p[f]);
            GridBar *gb = (GridBar *)fac->d_bar;
            int *err = fac->d_solve_err;
            T *scr = (T *)fac->d_coop_scratch;
            const int2 *units = fac->d_units + fac->unit_bwd_off[L];
            int nunits = fac->unit_bwd_n[L];
            unsigned bar_limit = bar_limit_of(fac), flag_limit = flag_limit_of(fac);
            void *args[] = {(void *)&fac->d_fronts, (void *)&fb, (void *)&nfl, (void *)&maxpp, (void *)&maxb,
                            (void *)&pool, (void *)&fac->d_vars, (void *)&x, (void *)&fac->d_coop_off,
                            (void *)&scr, (void *)&W, (void *)&Y, (void *)&sum_m, (void *)&n, (void *)&nrhs,
                            (void *)&gb, (void *)&err, (void *)&units, (void *)&nunits, (void *)&bar_limit,
                            (void *)&flag_limit};
            const int prw = (maxpp + kItemRows - 1) / kItemRows;
            const int cch = std::max(1, (maxb + kRowsPerCta - 1) / kRowsPerCta);
            const int items = std::max(std::max(nfl * prw * cch, nfl), nunits);
            const int grid = std::max(1, std::min(fac->coop_grid, items));
            CUDA_TRY(cudaLaunchCooperativeKernel(nrhs == 1 ? (const void *)k_bwd_level<T, R, 1> : (const void *)k_bwd_level<T, R, 8>, dim3(grid),
                                                 dim3(kRowsPerCta), args, sm_coop, st));
            prof_end(PROF_SOLVE_BWD, st, 1);
            continue;
        }
        if (warp_level_fits<T>(maxp, S.lev_max_m[L], nrhs)) {
            const int maxm = S.lev_max_m[L];
            k_bwd_warp<T><<<(nfl + kWarpFronts - 1) / kWarpFronts, 32 * kWarpFronts, warp_smem_bytes<T>(nrhs, maxm),
                            st>>>(fac->d_fronts, fac->d_vars, pool, Y, x, sum_m, n, nrhs, fb, nfl, maxm,
                                  (int)fac->blocked_level[L]);
            prof_end(PROF_SOLVE_BWD, st, 1);
            continue;
        }
        if (small_level_fits<T>(maxp, S.lev_max_m[L], nrhs)) {
            const int maxm = S.lev_max_m[L];
            k_bwd_small<T><<<nfl, kSmallThreads, small_smem_bytes<T>(nrhs, maxm), st>>>(
                fac->d_fronts, fac->d_vars, pool, Y, x, sum_m, n, nrhs, fb, maxm);
            prof_end(PROF_SOLVE_BWD, st, 1);
            continue;
        }
        int nbl = 1;
        if (fac->bwd_wide[L]) {
            int maxb = 0;
            for (int f = fb; f < fb + nfl; ++f) maxb = std::max(maxb, S.m[f] - S.p[f]);
            const int cch = (maxb + kRowsPerCta - 1) / kRowsPerCta;
            k_bwd_partial<T><<<dim3(nfl, prow, cch), kRowsPerCta, (size_t)nrhs * kRowsPerCta * sizeof(T),
                               st>>>(fac->d_fronts, pool, fac->d_vars, x, fac->d_bwd_off, (T *)fac->d_bwd_scratch,
                                     n, nrhs, fb);
            k_bwd_reduce<T><<<dim3(nfl, (maxp + kRowsPerCta - 1) / kRowsPerCta), kRowsPerCta, 0, st>>>(fac->d_fronts, fac->d_bwd_off,
                                                                    (const T *)fac->d_bwd_scratch, W, Y, sum_m,
                                                                    nrhs, fb);
            nbl = 2;
        } else {
            k_bwd_init<T><<<dim3(nfl, prow), kRowsPerCta, (size_t)nrhs * kRowsPerCta * sizeof(T), st>>>(
                fac->d_fronts, pool, fac->d_vars, W, Y, x, fac->d_unit, sum_m, n, nrhs, fb, fac->max_nrhs);
        }
        int nl = nbl;
        for (int k0 = ((maxp - 1) / NB) * NB; k0 >= 0; k0 -= NB, ++nl) {
            const int rows = std::max(1, (k0 + kItemRows - 1) / kItemRows);
            k_bwd_panel<T, R><<<dim3(nfl, rows), kRowsPerCta, sm_panel, st>>>(
                fac->d_fronts, pool, fac->d_vars, W, x, fac->d_unit, sum_m, n, nrhs, fb, k0);
        }
        prof_end(PROF_SOLVE_BWD, st, nl);
    }
    CUDA_TRY(cudaGetLastError());
    return FDFD_OK;
}

}  // namespace
}  // namespace fdfd

// The backward phase works in the scaled unknowns y = x / s_out; the global
// x written by k_bwd_panel must therefore stay in scaled units until every
// level is done (ancestors' x is read back by k_bwd_init).  The solve runs
// with unit scales internally and applies s_in / s_out around it.
namespace fdfd {
namespace {

// out[r] = s[r] in[r] for the nrhs columns of n entries.
__global__ void k_colscale(const double2 *in, double2 *out, const double *s, int64_t n, int nrhs) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        for (int r = 0; r < nrhs; ++r) {
            const double c = s[r];
            const double2 v = in[(size_t)r * n + k];
            out[(size_t)r * n + k] = make_double2(__dmul_rn(v.x, c), __dmul_rn(v.y, c));
        }
    }
}

// acc[r] += s[r] v[r], rounded as the scaling and the sum done apart.
__global__ void k_colscale_add(const double2 *v, double2 *acc, const double *s, int64_t n, int nrhs) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        for (int r = 0; r < nrhs; ++r) {
            const double c = s[r];
            const double2 a = acc[(size_t)r * n + k], b = v[(size_t)r * n + k];
            acc[(size_t)r * n + k] =
                make_double2(__dadd_rn(a.x, __dmul_rn(b.x, c)), __dadd_rn(a.y, __dmul_rn(b.y, c)));
        }
    }
}

// One application of the factor on device vectors (no host sync):
// out = A^-1 in  (transpose = 0) or A^-T in (transpose = 1).
// have_norms: fac->d_norm already holds the nrhs column norms of `in`
// (no transpose).  acc != NULL (no transpose): acc += A^-1 in instead, with
// `out` as the scratch of the solve.
int apply_factor(fdfd_factor *fac, const double2 *in, double2 *out, int nrhs, int transpose,
                 cudaStream_t st, bool have_norms = false, double2 *acc = nullptr) {
    const int64_t n = fac->n;
    if (transpose && !fac->has_p)
        return fail(FDFD_ERR_BAD_ARG, "transposed solve needs the operator's PML factors");
    double2 *tmp = fac->d_tmp;
    const double2 *src = in;
    if (transpose) {
        k_pscale<<<grid1(n * nrhs), 256, 0, st>>>(in, tmp, fac->d_isxf, fac->d_isyf, fac->Nx, fac->Ny,
                                                  nrhs, 0);
        src = tmp;
    }
    if (transpose) have_norms = false, acc = nullptr;
    // scales from the column norms of the right-hand side
    prof_begin(PROF_OTHER, st);
    int rc = have_norms ? FDFD_OK : norms_device(src, n, nrhs, fac->d_partial, fac->d_norm, st);
    if (rc) return rc;
    k_scales<<<1, 32, 0, st>>>(fac->d_norm, fac->d_maxdiag, nrhs, fac->d_sin, fac->d_sout);
    prof_end(PROF_OTHER, st, (have_norms ? 1 : 3) + (transpose ? 1 : 0));
    // the forward gathers read src scaled by s_in
    if (fac->precision != FDFD_PREC_C128)
        rc = solve_levels<c64, float>(fac, src, fac->d_sin, out, nrhs, st);
    else
        rc = solve_levels<c128, double>(fac, src, fac->d_sin, out, nrhs, st);
    if (rc) return rc;
    prof_begin(PROF_OTHER, st);
    if (acc)
        k_colscale_add<<<grid1(n), 256, 0, st>>>(out, acc, fac->d_sout, n, nrhs);
    else
        k_colscale<<<grid1(n), 256, 0, st>>>(out, out, fac->d_sout, n, nrhs);
    prof_end(PROF_OTHER, st, 1 + (transpose ? 1 : 0));
    if (transpose)
        k_pscale<<<grid1(n * nrhs), 256, 0, st>>>(out, out, fac->d_isxf, fac->d_isyf, fac->Nx, fac->Ny,
                                                  nrhs, 1);
    CUDA_TRY(cudaGetLastError());
    return FDFD_OK;
}

void free_factor(fdfd_factor *f) {
    if (f && f->graph) cudaGraphExecDestroy(f->graph);
    if (f && f->st_cap) cudaStreamDestroy(f->st_cap);
    if (!f) return;
    void *ptrs[] = {f->d_inv, f->d_piv, f->d_fronts, f->d_vars, f->d_relmap, f->d_nbr, f->d_vfront, f->d_vloc, f->d_pool,
                    f->d_W, f->d_Y, f->d_r, f->d_d, f->d_tmp, f->d_isxf, f->d_isyf, f->d_partial,
                    f->d_norm, f->d_sin, f->d_sout, f->d_unit, f->d_maxdiag, f->d_tiny,
                    f->d_tcf, f->d_scratch, f->d_tcerr, f->d_bwd_off, f->d_bwd_scratch,
                    f->d_bar, f->d_solve_err, f->d_coop_off, f->d_coop_scratch, f->d_krylov,
                    f->d_units, f->d_coef};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (f->h_norm) cudaFreeHost(f->h_norm);
    if (f->h_err) cudaFreeHost(f->h_err);
    for (auto &e : f->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : f->ev_look)
        if (e) cudaEventDestroy(e);
    if (f->st_look) cudaStreamDestroy(f->st_look);
    delete f;
}

// Tensor-core levels: fronts large enough for 128-row tiles to pay.
constexpr int kTcMinM = 192;

int64_t tc_layout(const Symbolic &S, std::vector<char> *lev, std::vector<TcFront> *tf) {
    int64_t best = 0;
    if (lev) lev->assign(S.nlev, 0);
    if (tf) tf->assign(S.nf, TcFront{});
    for (int L = 0; L < S.nlev; ++L) {
        if (S.lev_max_m[L] < kTcMinM) continue;
        if (lev) (*lev)[L] = 1;
        int64_t off = 0;
        for (int f = S.level_ptr[L]; f < S.level_ptr[L + 1]; ++f) {
            int64_t ab = 0;
            const int64_t tot = tc_front_scratch(S.m[f], S.p[f], &ab);
            if (tf) {
                (*tf)[f].a_off = off;
                (*tf)[f].b_off = off + ab;
            }
            off += tot;
        }
        best = std::max(best, off);
    }
    if (tf)
        for (int f = 0; f < S.nf; ++f) {
            (*tf)[f].f_off = S.pool_off[f];
            (*tf)[f].m = S.m[f];
            (*tf)[f].p = S.p[f];
            (*tf)[f].ld = S.ld[f];
        }
    return best;
}

// Levels whose fronts have a wide boundary use the two-pass backward
// opener; returns the scratch elements it needs (per-level maximum).
constexpr int kBwdWide = 512;
int64_t bwd_layout(const Symbolic &S, int max_nrhs, std::vector<char> *wide, std::vector<int64_t> *off) {
    int64_t best = 0;
    if (wide) wide->assign(S.nlev, 0);
    if (off) off->assign(S.nf, 0);
    for (int L = 0; L < S.nlev; ++L) {
        int maxb = 0;
        for (int f = S.level_ptr[L]; f < S.level_ptr[L + 1]; ++f) maxb = std::max(maxb, S.m[f] - S.p[f]);
        if (maxb < kBwdWide) continue;
        if (wide) (*wide)[L] = 1;
        int64_t o = 0;
        for (int f = S.level_ptr[L]; f < S.level_ptr[L + 1]; ++f) {
            if (off) (*off)[f] = o;
            const int64_t nch = (S.m[f] - S.p[f] + kRowsPerCta - 1) / kRowsPerCta;
            o += nch * max_nrhs * (int64_t)S.p[f];
        }
        best = std::max(best, o);
    }
    return best;
}

// Levels with at least kCoopPanels panel steps run their substitutions as
// cooperative launches; their opener scratch (per front: column blocks x
// rhs x p) is laid out here.
constexpr int kCoopPanels = 2;
int64_t coop_layout(const Symbolic &S, int max_nrhs, std::vector<char> *lev, std::vector<int64_t> *off) {
    int64_t best = 0;
    if (lev) lev->assign(S.nlev, 0);
    if (off) off->assign(S.nf, 0);
    for (int L = 0; L < S.nlev; ++L) {
        if ((S.lev_max_p[L] + NB - 1) / NB < kCoopPanels) continue;
        if (lev) (*lev)[L] = 1;
        int64_t o = 0;
        for (int f = S.level_ptr[L]; f < S.level_ptr[L + 1]; ++f) {
            if (off) (*off)[f] = o;
            const int64_t nch = std::max<int64_t>(1, (S.m[f] - S.p[f] + kRowsPerCta - 1) / kRowsPerCta);
            o += nch * max_nrhs * (int64_t)S.p[f];
        }
        best = std::max(best, o);
    }
    return best;
}

// Work units of the pipelined substitutions on the cooperative levels, one
// per (front, block of up to 64 rows).  Forward list: pivot blocks R < KP
// (rows [64R, min(64R + 64, p))) and update-row blocks numbered KP, KP+1, ...
// (rows p + 64 (R - KP) ...), sorted by R; backward list: pivot blocks sorted
// by KP - 1 - R.  A unit waits only on units of its own front that come
// earlier in its list, so CTAs that take the units in list order (all CTAs
// co-resident) always make progress.
struct PipeLayout {
    std::vector<int2> units;
    std::vector<int> fwd_off, fwd_n, bwd_off, bwd_n;
};
PipeLayout pipe_layout(const Symbolic &S) {
    PipeLayout pl;
    pl.fwd_off.assign(S.nlev, 0);
    pl.fwd_n.assign(S.nlev, 0);
    pl.bwd_off.assign(S.nlev, 0);
    pl.bwd_n.assign(S.nlev, 0);
    for (int L = 0; L < S.nlev; ++L) {
        const int kpm = (S.lev_max_p[L] + NB - 1) / NB;
        if (kpm < kCoopPanels) continue;
        const int fb = S.level_ptr[L], nfl = S.level_ptr[L + 1] - fb;
        int rmax = 0;
        for (int f = fb; f < fb + nfl; ++f)
            rmax = std::max(rmax, (S.p[f] + NB - 1) / NB + (S.m[f] - S.p[f] + NB - 1) / NB);
        pl.fwd_off[L] = (int)pl.units.size();
        for (int R = 0; R < rmax; ++R)
            for (int f = fb; f < fb + nfl; ++f) {
                const int kp = (S.p[f] + NB - 1) / NB, kb = (S.m[f] - S.p[f] + NB - 1) / NB;
                if (R < kp + kb) pl.units.push_back(make_int2(f - fb, R));
            }
        pl.fwd_n[L] = (int)pl.units.size() - pl.fwd_off[L];
        pl.bwd_off[L] = (int)pl.units.size();
        for (int d = 0; d < kpm; ++d)
            for (int f = fb; f < fb + nfl; ++f) {
                const int kp = (S.p[f] + NB - 1) / NB;
                if (d < kp) pl.units.push_back(make_int2(f - fb, kp - 1 - d));
            }
        pl.bwd_n[L] = (int)pl.units.size() - pl.bwd_off[L];
    }
    return pl;
}

int64_t factor_bytes_of(const Symbolic &S, int precision, int max_nrhs) {
    const int64_t elem = precision == FDFD_PREC_C128 ? 16 : 8;
    const int64_t n = (int64_t)S.Nx * S.Ny;
    int64_t b = S.pool_entries * elem;
    b += 2 * S.sum_m * max_nrhs * elem;                  // W, Y
    b += 3 * n * max_nrhs * 16;                          // r, d, tmp
    b += (int64_t)S.nf * sizeof(FrontD);
    b += 4 * S.sum_m * 4 + 7 * n * 4;                    // vars, relmap, inverse maps, nbr, var maps, pivots
    b += (int64_t)(S.Nx + S.Ny) * 16;
    b += 5 * n * 16;                                     // operator coefficients
    b += (int64_t)norms_partial_count(max_nrhs * S.batch) * 8 + 4 * max_nrhs * S.batch * 8 + 64;
    if (precision == FDFD_PREC_C64_TC) b += tc_layout(S, nullptr, nullptr) + (int64_t)S.nf * sizeof(TcFront);
    b += bwd_layout(S, max_nrhs, nullptr, nullptr) * elem + (int64_t)S.nf * 8;
    b += coop_layout(S, max_nrhs, nullptr, nullptr) * elem + (int64_t)S.nf * 8 + 16;
    const PipeLayout pl = pipe_layout(S);
    b += (int64_t)pl.units.size() * sizeof(int2);
    return b;
}

}  // namespace
}  // namespace fdfd

template <typename T, typename R>
int coop_grid_for(int max_nrhs, int *grid) {
    int dev = 0, sms = 0, coop = 0, nb1 = 0, nb2 = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) {
        *grid = 0;
        return FDFD_OK;
    }
    const size_t smem = std::max(panel_smem_bytes<T>(max_nrhs), (size_t)max_nrhs * kRowsPerCta * sizeof(T));
    int nb3 = 0, nb4 = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, k_fwd_level<T, R, 8>, kRowsPerCta, smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, k_bwd_level<T, R, 8>, kRowsPerCta, smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb3, k_fwd_level<T, R, 1>, kRowsPerCta, smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb4, k_bwd_level<T, R, 1>, kRowsPerCta, smem));
    const int per_sm = std::min(std::min(std::min(nb1, nb2), std::min(nb3, nb4)), 4);
    *grid = per_sm > 0 ? per_sm * sms : 0;
    return FDFD_OK;
}

extern "C" int fdfd_factor_bytes(const fdfd_symbolic *sym, int32_t precision, int32_t max_nrhs,
                                 int64_t *bytes) {
    if (!sym || !bytes) return fail(FDFD_ERR_BAD_ARG, "factor_bytes: NULL argument");
    if (precision != FDFD_PREC_C128 && precision != FDFD_PREC_C64 && precision != FDFD_PREC_C64_TC)
        return fail(FDFD_ERR_BAD_ARG, "factor_bytes: unknown precision");
    if (max_nrhs < 1 || max_nrhs > 8) return fail(FDFD_ERR_BAD_ARG, "factor_bytes: max_nrhs must be 1..8");
    *bytes = factor_bytes_of(sym->s, precision, max_nrhs);
    return FDFD_OK;
}

extern "C" int fdfd_factor_create(fdfd_symbolic *sym, int32_t precision, int32_t max_nrhs,
                                  fdfd_factor **out) {
    if (!sym || !out) return fail(FDFD_ERR_BAD_ARG, "factor_create: NULL argument");
    *out = nullptr;
    if (precision != FDFD_PREC_C128 && precision != FDFD_PREC_C64 && precision != FDFD_PREC_C64_TC)
        return fail(FDFD_ERR_BAD_ARG, "factor_create: unknown precision");
    if (max_nrhs < 1 || max_nrhs > 8) return fail(FDFD_ERR_BAD_ARG, "factor_create: max_nrhs must be 1..8");
    const Symbolic &S = sym->s;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail(FDFD_ERR_NO_DEVICE, "factor_create: no CUDA device");
    }
    fdfd_factor *f = new fdfd_factor();
    f->sym = sym;
    f->precision = precision;
    f->max_nrhs = max_nrhs;
    f->elem = precision == FDFD_PREC_C128 ? 16 : 8;
    f->use_tc = precision == FDFD_PREC_C64_TC;
    f->n = (int64_t)S.Nx * S.Ny;
    f->Nx = S.Nx;
    f->Ny = S.Ny;
    f->batch = S.batch;
    f->rows = S.rows;
    const int nseg = max_nrhs * S.batch;  // norm segments: right-hand side x problem
    cudaGetDevice(&f->device);

    std::vector<FrontD> fd(S.nf);
    for (int i = 0; i < S.nf; ++i) {
        fd[i].f_off = S.pool_off[i];
        fd[i].m = S.m[i];
        fd[i].p = S.p[i];
        fd[i].ld = S.ld[i];
        fd[i].voff = S.vars_off[i];
        fd[i].c0 = S.child0[i];
        fd[i].c1 = S.child1[i];
    }
    auto alloc = [&](void **p, size_t bytes) -> bool {
        cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return true;
    };
    const int64_t n = f->n;
    bool ok = alloc((void **)&f->d_fronts, S.nf * sizeof(FrontD)) &&
              alloc((void **)&f->d_vars, S.sum_m * 4) && alloc((void **)&f->d_relmap, S.sum_m * 4) &&
              alloc((void **)&f->d_inv, 2 * S.sum_m * 4) && alloc((void **)&f->d_piv, n * 4) &&
              alloc((void **)&f->d_nbr, 4 * n * 4) && alloc((void **)&f->d_vfront, n * 4) &&
              alloc((void **)&f->d_vloc, n * 4) && alloc(&f->d_pool, S.pool_entries * f->elem) &&
              alloc(&f->d_W, S.sum_m * max_nrhs * f->elem) &&
              alloc(&f->d_Y, S.sum_m * max_nrhs * f->elem) &&
              alloc((void **)&f->d_r, n * max_nrhs * 16) && alloc((void **)&f->d_d, n * max_nrhs * 16) &&
              alloc((void **)&f->d_tmp, n * max_nrhs * 16) && alloc((void **)&f->d_isxf, S.Nx * 16) &&
              alloc((void **)&f->d_isyf, S.Ny * 16) &&
              alloc((void **)&f->d_partial, norms_partial_count(nseg) * 8) &&
              alloc((void **)&f->d_norm, nseg * 8) && alloc((void **)&f->d_sin, max_nrhs * 8) &&
              alloc((void **)&f->d_sout, max_nrhs * 8) && alloc((void **)&f->d_unit, 8 * 8) &&
              alloc((void **)&f->d_maxdiag, 8) && alloc((void **)&f->d_tiny, 4) &&
              alloc((void **)&f->d_coef, 5 * n * 16);
    if (!ok) {
        free_factor(f);
        return fail(FDFD_ERR_OOM, "factor_create: device allocation failed");
    }
    cudaError_t e = cudaMallocHost((void **)&f->h_norm, std::max(8, nseg) * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&f->h_err, sizeof(int));
    for (auto &ev : f->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    const double ones[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    if (e == cudaSuccess) e = cudaMemcpy(f->d_fronts, fd.data(), S.nf * sizeof(FrontD), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_vars, S.vars.data(), S.sum_m * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_relmap, S.relmap.data(), S.sum_m * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        // inverse of the children's row maps, for the parent-side extend-add
        std::vector<int32_t> inv((size_t)2 * S.sum_m, -1);
        for (int32_t c = 0; c < S.nf; ++c) {
            const int32_t par = S.parent[c];
            if (par < 0) continue;
            const int64_t base = (S.child0[par] == c ? 0 : S.sum_m) + S.vars_off[par];
            for (int32_t k = S.p[c]; k < S.m[c]; ++k) inv[base + S.relmap[S.vars_off[c] + k]] = k - S.p[c];
        }
        e = cudaMemcpy(f->d_inv, inv.data(), inv.size() * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        std::vector<int32_t> piv;
        piv.reserve(n);
        f->piv_off.assign(S.nlev + 1, 0);
        for (int L = 0; L < S.nlev; ++L) {
            for (int32_t fr = S.level_ptr[L]; fr < S.level_ptr[L + 1]; ++fr)
                for (int32_t k = 0; k < S.p[fr]; ++k) piv.push_back(S.vars[S.vars_off[fr] + k]);
            f->piv_off[L + 1] = (int64_t)piv.size();
        }
        e = cudaMemcpy(f->d_piv, piv.data(), piv.size() * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(f->d_nbr, S.nbr_loc.data(), 4 * n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_vfront, S.var_front.data(), n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_vloc, S.var_loc.data(), n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_unit, ones, sizeof(ones), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_factor(f);
        return fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
    }
    int rc = (precision != FDFD_PREC_C128) ? set_smem_attrs<c64, float>() : set_smem_attrs<c128, double>();
    if (rc == FDFD_OK && f->use_tc) {
        std::vector<TcFront> tf;
        const int64_t sb = tc_layout(S, &f->tc_level, &tf);
        if (!alloc((void **)&f->d_tcf, S.nf * sizeof(TcFront)) || !alloc((void **)&f->d_scratch, sb) ||
            !alloc((void **)&f->d_tcerr, 4)) {
            free_factor(f);
            return fail(FDFD_ERR_OOM, "factor_create: tensor-core scratch allocation failed");
        }
        e = cudaMemcpy(f->d_tcf, tf.data(), S.nf * sizeof(TcFront), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(f->d_tcerr, 0, 4);
        if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
        if (rc == FDFD_OK) rc = tc_prepare();
        if (rc == FDFD_OK) {
            int lo = 0, hi = 0;
            e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&f->st_look, cudaStreamNonBlocking, hi);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_look[0], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_look[1], cudaEventDisableTiming);
            if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
        }
    }
    if (rc == FDFD_OK) {
        std::vector<int64_t> coff;
        const int64_t ce = coop_layout(S, max_nrhs, &f->coop_level, &coff);
        rc = (precision != FDFD_PREC_C128) ? coop_grid_for<c64, float>(max_nrhs, &f->coop_grid)
                                           : coop_grid_for<c128, double>(max_nrhs, &f->coop_grid);
        if (rc == FDFD_OK && f->coop_grid == 0) f->coop_level.assign(S.nlev, 0);  // no cooperative launch
        if (rc == FDFD_OK) {
            int dev = 0, sms = 0, per_sm = 0;
            e = cudaGetDevice(&dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_coef, kCoefCols, 0);
            if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
            else f->coef_ctas = std::max(1, sms * per_sm);
        }
        if (rc == FDFD_OK &&
            (!alloc(&f->d_bar, sizeof(GridBar)) || !alloc((void **)&f->d_solve_err, 4) ||
             !alloc((void **)&f->d_coop_off, S.nf * sizeof(int64_t)) || !alloc(&f->d_coop_scratch, ce * f->elem))) {
            free_factor(f);
            return fail(FDFD_ERR_OOM, "factor_create: cooperative-solve scratch allocation failed");
        }
        if (rc == FDFD_OK) {
            e = cudaMemcpy(f->d_coop_off, coff.data(), S.nf * sizeof(int64_t), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemset(f->d_solve_err, 0, 4);
            if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
        }
        if (rc == FDFD_OK) {
            PipeLayout pl = pipe_layout(S);
            f->unit_fwd_off = pl.fwd_off;
            f->unit_fwd_n = pl.fwd_n;
            f->unit_bwd_off = pl.bwd_off;
            f->unit_bwd_n = pl.bwd_n;
            if (!alloc((void **)&f->d_units, pl.units.size() * sizeof(int2))) {
                free_factor(f);
                return fail(FDFD_ERR_OOM, "factor_create: pipelined-solve allocation failed");
            }
            e = cudaMemcpy(f->d_units, pl.units.data(), pl.units.size() * sizeof(int2), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
        }
    }
    if (rc == FDFD_OK) {
        std::vector<int64_t> boff;
        const int64_t be = bwd_layout(S, max_nrhs, &f->bwd_wide, &boff);
        if (!alloc((void **)&f->d_bwd_off, S.nf * sizeof(int64_t)) || !alloc(&f->d_bwd_scratch, be * f->elem)) {
            free_factor(f);
            return fail(FDFD_ERR_OOM, "factor_create: backward-solve scratch allocation failed");
        }
        e = cudaMemcpy(f->d_bwd_off, boff.data(), S.nf * sizeof(int64_t), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("factor_create: ") + cudaGetErrorString(e));
    }
    if (rc) {
        free_factor(f);
        return rc;
    }
    *out = f;
    return FDFD_OK;
}

extern "C" int fdfd_factor_set_pivot_tol(fdfd_factor *fac, double rel_tol) {
    if (!fac) return fail(FDFD_ERR_BAD_ARG, "factor_set_pivot_tol: NULL factor");
    if (!(rel_tol >= 0.0) && rel_tol != -1.0)
        return fail(FDFD_ERR_BAD_ARG, "factor_set_pivot_tol: tolerance must be >= 0 (or -1 for the default)");
    fac->pivot_tol = rel_tol;
    return FDFD_OK;
}

extern "C" int fdfd_factor_set_fused_limit(fdfd_factor *fac, int32_t max_m) {
    if (!fac) return fail(FDFD_ERR_BAD_ARG, "factor_set_fused_limit: NULL factor");
    if (max_m < -1) return fail(FDFD_ERR_BAD_ARG, "factor_set_fused_limit: max_m must be >= -1");
    fac->fused_max_m = max_m;
    return FDFD_OK;
}

// The refinement residual of an operator that is the factored one (same
// description: grid, scalars and device buffers) reads the coefficients
// stored at fdfd_factor_numeric.
static bool same_operator(const fdfd_operator &a, const fdfd_operator &b) {
    return a.Nx == b.Nx && a.Ny == b.Ny && a.pol == b.pol && a.averaging == b.averaging && a.omega == b.omega &&
           a.L0 == b.L0 && a.xlen == b.xlen && a.ylen == b.ylen && a.eps == b.eps && a.eps_add == b.eps_add &&
           a.diag_add == b.diag_add && a.inv_sxf == b.inv_sxf && a.inv_sxb == b.inv_sxb &&
           a.inv_syf == b.inv_syf && a.inv_syb == b.inv_syb && a.stencil == b.stencil;
}
static void use_stored_coefficients(const fdfd_factor *fac, const fdfd_operator *op, OpDev *o) {
    if (fac->coef_valid && !o->stencil && same_operator(*op, fac->coef_op)) o->stencil = fac->d_coef;
}

extern "C" int fdfd_factor_numeric(fdfd_factor *fac, const fdfd_operator *op, void *stream) {
    if (!fac) return fail(FDFD_ERR_BAD_ARG, "factor_numeric: NULL factor");
    if (fac->batch > 1) return fail(FDFD_ERR_BAD_ARG, "factor_numeric: a batch factor takes fdfd_factor_numeric_batch");
    OpDev o;
    int rc = make_opdev(op, &o);
    if (rc) return rc;
    if (op->Nx != fac->Nx || op->Ny != fac->Ny)
        return fail(FDFD_ERR_BAD_ARG, "factor_numeric: operator grid differs from the symbolic grid");
    cudaStream_t st = (cudaStream_t)stream;
    fac->has_p = op->inv_sxf && op->inv_syf;
    if (fac->has_p) {
        CUDA_TRY(cudaMemcpyAsync(fac->d_isxf, op->inv_sxf, fac->Nx * 16, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(fac->d_isyf, op->inv_syf, fac->Ny * 16, cudaMemcpyDeviceToDevice, st));
    }
    CUDA_TRY(cudaEventRecord(fac->ev[0], st));
    fac->coef_valid = false;
    if (!o.stencil) {
        prof_begin(PROF_ASSEMBLE, st);
        coef_launch(o, fac->d_coef, fac->n, fac->coef_ctas, st);
        prof_end(PROF_ASSEMBLE, st, 1);
        o.stencil = fac->d_coef;
    }
    rc = (fac->precision != FDFD_PREC_C128) ? factor_levels_graphed<c64, float>(fac, o, st)
                                            : factor_levels_graphed<c128, double>(fac, o, st);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(fac->ev[1], st));
    fac->coef_op = *op;
    fac->coef_valid = !op->stencil;
    if (fac->d_tcerr) {
        // a bounded wait of the tensor-core Schur update that ran out left
        // tiles without their update: the factor is not valid
        CUDA_TRY(cudaMemcpyAsync(fac->h_err, fac->d_tcerr, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (*fac->h_err) {
            fac->numeric_done = false;
            return fail(FDFD_ERR_TIMEOUT, "factor_numeric: a bounded wait of the tensor-core Schur update ran out "
                                          "(the factor is not valid)");
        }
    }
    fac->numeric_done = true;
    return FDFD_OK;
}

extern "C" int fdfd_factor_solve(fdfd_factor *fac, const void *b, void *x, int32_t nrhs,
                                 int32_t transpose, void *stream) {
    if (!fac || !b || !x) return fail(FDFD_ERR_BAD_ARG, "factor_solve: NULL argument");
    if (!fac->numeric_done) return fail(FDFD_ERR_BAD_ARG, "factor_solve: factor has no numeric values");
    if (nrhs < 1 || nrhs > fac->max_nrhs) return fail(FDFD_ERR_BAD_ARG, "factor_solve: nrhs out of range");
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaEventRecord(fac->ev[2], st));
    CUDA_TRY(cudaMemsetAsync(fac->d_solve_err, 0, sizeof(int), st));
    int rc = apply_factor(fac, (const double2 *)b, (double2 *)x, nrhs, transpose, st);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(fac->ev[3], st));
    // the cooperative substitutions report a bounded wait that ran out in
    // d_solve_err: read it (one synchronisation of the stream)
    CUDA_TRY(cudaMemcpyAsync(fac->h_err, fac->d_solve_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (*fac->h_err)
        return fail(FDFD_ERR_TIMEOUT, "factor_solve: a bounded wait of the cooperative substitutions ran out (the "
                                      "solution is not valid)");
    return FDFD_OK;
}

extern "C" int fdfd_factor_set_graphs(fdfd_factor *fac, int32_t on) {
    if (!fac) return fail(FDFD_ERR_BAD_ARG, "factor_set_graphs: NULL factor");
    fac->use_graphs = on != 0;
    if (!fac->use_graphs && fac->graph) {
        cudaGraphExecDestroy(fac->graph);
        fac->graph = nullptr;
    }
    return FDFD_OK;
}

extern "C" int fdfd_factor_set_wait_limit(fdfd_factor *fac, int64_t polls) {
    if (!fac) return fail(FDFD_ERR_BAD_ARG, "factor_set_wait_limit: NULL factor");
    if (polls < 1 && polls != -1)
        return fail(FDFD_ERR_BAD_ARG, "factor_set_wait_limit: polls must be >= 1 (or -1 for the default)");
    fac->wait_limit = polls < 0 ? 0 : polls;
    return FDFD_OK;
}

// FP64 iterative refinement shared by the single and the batch entry
// points: x = M^-1 b, then x += M^-1 (b - A x) until every one of the nseg
// segments (seg entries each: a right-hand side of one problem) has
// ||b - A x|| <= tol ||b|| or max_iter steps were taken.  seg_rel (host,
// nseg doubles, optional) receives the final relative residuals.
static int refine_loop(fdfd_factor *fac, const OpDev &o, const double2 *bb, double2 *xx, int nrhs,
                       int transpose, double tol, int max_iter, int64_t seg, int nseg, double *seg_rel,
                       const char *who, cudaStream_t st) {
    const int64_t n = fac->n;
    CUDA_TRY(cudaEventRecord(fac->ev[2], st));
    CUDA_TRY(cudaMemsetAsync(fac->d_solve_err, 0, sizeof(int), st));
    std::vector<double> bnorm(nseg);
    prof_begin(PROF_OTHER, st);
    int rc = norms_device(bb, seg, nseg, fac->d_partial, fac->d_norm, st);
    if (rc) return rc;
    prof_end(PROF_OTHER, st, 2);
    CUDA_TRY(cudaMemcpyAsync(fac->h_norm, fac->d_norm, nseg * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int r = 0; r < nseg; ++r) bnorm[r] = fac->h_norm[r];
    rc = apply_factor(fac, bb, xx, nrhs, transpose, st);
    if (rc) return rc;
    double worst = 0.0;
    int it = 0;
    for (;;) {
        // r = b - A x (or b - A^T x), FP64, matrix-free
        prof_begin(PROF_OTHER, st);
        rc = apply_device(o, xx, bb, fac->d_r, nrhs, transpose ? 3 : 0, st);
        if (rc) return rc;
        rc = norms_device(fac->d_r, seg, nseg, fac->d_partial, fac->d_norm, st);
        if (rc) return rc;
        prof_end(PROF_OTHER, st, 3);
        CUDA_TRY(cudaMemcpyAsync(fac->h_norm, fac->d_norm, nseg * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(fac->h_err, fac->d_solve_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (*fac->h_err)
            return fail(FDFD_ERR_TIMEOUT, std::string(who) + ": a bounded wait of the cooperative substitutions "
                                                              "ran out (the solution is not valid)");
        worst = 0.0;
        for (int r = 0; r < nseg; ++r) {
            const double rel = bnorm[r] > 0 ? fac->h_norm[r] / bnorm[r] : fac->h_norm[r];
            if (seg_rel) seg_rel[r] = rel;
            worst = std::max(worst, rel);
        }
        if (!(worst > tol) || it >= max_iter) break;
        // x += M^-1 r: d_norm holds the residual's column norms when the
        // segments are the columns; the correction is added by the
        // solve's final scaling (no transpose)
        if (transpose) {
            rc = apply_factor(fac, fac->d_r, fac->d_d, nrhs, transpose, st);
            if (rc) return rc;
            prof_begin(PROF_OTHER, st);
            k_axpy<<<grid1(n * nrhs), 256, 0, st>>>(xx, fac->d_d, n * nrhs);
            prof_end(PROF_OTHER, st, 1);
        } else {
            rc = apply_factor(fac, fac->d_r, fac->d_d, nrhs, 0, st, seg == n && nseg == nrhs, xx);
            if (rc) return rc;
        }
        ++it;
    }
    CUDA_TRY(cudaEventRecord(fac->ev[3], st));
    fac->stats.refine_iters = it;
    fac->stats.rel_residual = worst;
    if (!(worst <= tol))
        return fail(FDFD_ERR_NOT_CONVERGED, std::string(who) + ": residual " + std::to_string(worst) +
                                                " above tolerance after " + std::to_string(it) +
                                                " refinement steps");
    return FDFD_OK;
}

extern "C" int fdfd_solve_refined(fdfd_factor *fac, const fdfd_operator *op, const void *b, void *x,
                                  int32_t nrhs, int32_t transpose, double tol, int32_t max_iter,
                                  void *stream) {
    if (!fac || !b || !x) return fail(FDFD_ERR_BAD_ARG, "solve_refined: NULL argument");
    if (!fac->numeric_done) return fail(FDFD_ERR_BAD_ARG, "solve_refined: factor has no numeric values");
    if (fac->batch > 1) return fail(FDFD_ERR_BAD_ARG, "solve_refined: a batch factor takes fdfd_solve_refined_batch");
    if (nrhs < 1 || nrhs > fac->max_nrhs) return fail(FDFD_ERR_BAD_ARG, "solve_refined: nrhs out of range");
    if (max_iter < 0) return fail(FDFD_ERR_BAD_ARG, "solve_refined: max_iter must be >= 0");
    OpDev o;
    int rc = make_opdev(op, &o);
    if (rc) return rc;
    if (op->Nx != fac->Nx || op->Ny != fac->Ny)
        return fail(FDFD_ERR_BAD_ARG, "solve_refined: operator grid differs from the factor grid");
    use_stored_coefficients(fac, op, &o);
    return refine_loop(fac, o, (const double2 *)b, (double2 *)x, nrhs, transpose, tol, max_iter, fac->n, nrhs,
                       nullptr, "solve_refined", (cudaStream_t)stream);
}

// ---- batches: one forest factorization of `batch` same-grid operators -------
// The operators' coefficients are evaluated into consecutive slices of the
// factor's coefficient store; from then on the forest is one explicit-
// stencil operator of batch * rows rows whose wrap stays inside each
// problem's rows (OpDev::Nxp), so every level's launches cover the fronts
// of all problems and the refinement residual of all problems is one pass.
static OpDev batch_opdev(const fdfd_factor *fac) {
    OpDev o{};
    o.Nx = fac->Nx;
    o.Ny = fac->Ny;
    o.Nxp = fac->rows;
    o.stencil = fac->d_coef;
    return o;
}

extern "C" int fdfd_factor_numeric_batch(fdfd_factor *fac, const fdfd_operator *ops, int32_t count,
                                         void *stream) {
    if (!fac || !ops) return fail(FDFD_ERR_BAD_ARG, "factor_numeric_batch: NULL argument");
    if (count != fac->batch)
        return fail(FDFD_ERR_BAD_ARG, "factor_numeric_batch: count must equal the symbolic's batch (" +
                                          std::to_string(fac->batch) + ")");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n1 = (int64_t)fac->rows * fac->Ny;
    CUDA_TRY(cudaEventRecord(fac->ev[0], st));
    for (int b = 0; b < count; ++b) {
        OpDev o;
        int rc = make_opdev(&ops[b], &o);
        if (rc) return rc;
        if (ops[b].Nx != fac->rows || ops[b].Ny != fac->Ny)
            return fail(FDFD_ERR_BAD_ARG, "factor_numeric_batch: operator " + std::to_string(b) +
                                              " differs from the batch's grid");
        prof_begin(PROF_ASSEMBLE, st);
        coef_launch(o, fac->d_coef + b * n1, fac->n, fac->coef_ctas, st);
        prof_end(PROF_ASSEMBLE, st, 1);
    }
    fac->has_p = false;
    fac->coef_valid = false;
    const OpDev o = batch_opdev(fac);
    int rc = (fac->precision != FDFD_PREC_C128) ? factor_levels_graphed<c64, float>(fac, o, st)
                                                : factor_levels_graphed<c128, double>(fac, o, st);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(fac->ev[1], st));
    if (fac->d_tcerr) {
        CUDA_TRY(cudaMemcpyAsync(fac->h_err, fac->d_tcerr, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (*fac->h_err) {
            fac->numeric_done = false;
            return fail(FDFD_ERR_TIMEOUT, "factor_numeric_batch: a bounded wait of the tensor-core Schur update "
                                          "ran out (the factor is not valid)");
        }
    }
    fac->numeric_done = true;
    return FDFD_OK;
}

extern "C" int fdfd_solve_refined_batch(fdfd_factor *fac, const void *b, void *x, int32_t nrhs, double tol,
                                        int32_t max_iter, double *rel_residuals, void *stream) {
    if (!fac || !b || !x) return fail(FDFD_ERR_BAD_ARG, "solve_refined_batch: NULL argument");
    if (!fac->numeric_done) return fail(FDFD_ERR_BAD_ARG, "solve_refined_batch: factor has no numeric values");
    if (nrhs < 1 || nrhs > fac->max_nrhs) return fail(FDFD_ERR_BAD_ARG, "solve_refined_batch: nrhs out of range");
    if (max_iter < 0) return fail(FDFD_ERR_BAD_ARG, "solve_refined_batch: max_iter must be >= 0");
    const OpDev o = batch_opdev(fac);
    const int64_t n1 = (int64_t)fac->rows * fac->Ny;
    return refine_loop(fac, o, (const double2 *)b, (double2 *)x, nrhs, 0, tol, max_iter, n1, nrhs * fac->batch,
                       rel_residuals, "solve_refined_batch", (cudaStream_t)stream);
}

// Right-preconditioned restarted GMRES in FP64 with the factor as the
// preconditioner M ~ A: x = x0 + M^-1 V y.  Arnoldi with two passes of
// classical Gram-Schmidt (batched dot products, one host round trip per
// pass), Givens rotations on the host.  Refinement by GMRES converges in
// fewer factor applications than plain refinement when the factor is only
// FP32 accurate.
extern "C" int fdfd_solve_gmres(fdfd_factor *fac, const fdfd_operator *op, const void *b, void *x,
                                int32_t transpose, double tol, int32_t max_iter, int32_t restart,
                                void *stream) {
    if (!fac || !b || !x) return fail(FDFD_ERR_BAD_ARG, "solve_gmres: NULL argument");
    if (!fac->numeric_done) return fail(FDFD_ERR_BAD_ARG, "solve_gmres: factor has no numeric values");
    if (fac->batch > 1) return fail(FDFD_ERR_BAD_ARG, "solve_gmres: not available for a batch factor");
    if (restart < 1 || restart > 30 || max_iter < 0) return fail(FDFD_ERR_BAD_ARG, "solve_gmres: restart must be 1..30");
    OpDev o;
    int rc = make_opdev(op, &o);
    if (rc) return rc;
    if (op->Nx != fac->Nx || op->Ny != fac->Ny)
        return fail(FDFD_ERR_BAD_ARG, "solve_gmres: operator grid differs from the factor grid");
    use_stored_coefficients(fac, op, &o);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = fac->n;
    const int m = restart;
    const int mode_apply = transpose ? 2 : 1, mode_res = transpose ? 3 : 0;
    const double2 *bb = (const double2 *)b;
    double2 *xx = (double2 *)x;
    // workspace: V (m+1 vectors), Z (m vectors), w; partial sums; coefficients
    if (!fac->d_krylov || fac->krylov_m < m) {
        if (fac->d_krylov) cudaFree(fac->d_krylov);
        fac->d_krylov = nullptr;
        const size_t bytes = (size_t)(2 * m + 2) * n * sizeof(double2) + (size_t)(m + 2) * kDotParts * sizeof(double2) +
                             64 * sizeof(double2);
        if (cudaMalloc(&fac->d_krylov, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(FDFD_ERR_OOM, "solve_gmres: Krylov workspace allocation failed");
        }
        fac->krylov_m = m;
    }
    double2 *V = (double2 *)fac->d_krylov;
    double2 *Z = V + (size_t)(m + 1) * n;
    double2 *w = Z + (size_t)m * n;
    double2 *partial = w + n;
    double2 *coef = partial + (size_t)(m + 2) * kDotParts;
    std::vector<double2> hcoef(m + 2);
    CUDA_TRY(cudaEventRecord(fac->ev[2], st));
    CUDA_TRY(cudaMemsetAsync(fac->d_solve_err, 0, sizeof(int), st));
    auto dots = [&](int nv, const double2 *vec) -> int {  // hcoef[0:nv] = V[0:nv]^H vec
        k_multidot_partial<<<dim3(kDotParts, nv), 256, 0, st>>>(V, n, nv, vec, partial);
        k_multidot_final<<<nv, 256, 0, st>>>(partial, kDotParts, coef);
        CUDA_TRY(cudaMemcpyAsync(hcoef.data(), coef, nv * sizeof(double2), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return FDFD_OK;
    };
    auto norm_of = [&](const double2 *vec, double *out) -> int {
        int r2 = norms_device(vec, n, 1, fac->d_partial, fac->d_norm, st);
        if (r2) return r2;
        CUDA_TRY(cudaMemcpyAsync(fac->h_norm, fac->d_norm, sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        *out = fac->h_norm[0];
        return FDFD_OK;
    };
    double bnorm = 0.0;
    if ((rc = norm_of(bb, &bnorm))) return rc;
    if (bnorm == 0.0) {
        CUDA_TRY(cudaMemsetAsync(xx, 0, n * sizeof(double2), st));
        fac->stats.refine_iters = 0;
        fac->stats.rel_residual = 0.0;
        return FDFD_OK;
    }
    // x0 = M^-1 b
    if ((rc = apply_factor(fac, bb, xx, 1, transpose, st))) return rc;
    int apps = 1;
    double rel = 0.0;
    std::vector<std::complex<double>> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    for (;;) {
        // r = b - A x into V[0]
        if ((rc = apply_device(o, xx, bb, V, 1, mode_res, st))) return rc;
        double beta = 0.0;
        if ((rc = norm_of(V, &beta))) return rc;
        rel = beta / bnorm;
        if (!(rel > tol) || apps > max_iter) break;
        k_scale_copy<<<grid1(n), 256, 0, st>>>(V, V, n, 1.0 / beta);
        std::fill(g.begin(), g.end(), std::complex<double>(0.0));
        g[0] = beta;
        int j = 0;
        for (; j < m && apps <= max_iter; ++j) {
            double2 *vj = V + (size_t)j * n, *zj = Z + (size_t)j * n;
            if ((rc = apply_factor(fac, vj, zj, 1, transpose, st))) return rc;
            ++apps;
            if ((rc = apply_device(o, zj, nullptr, w, 1, mode_apply, st))) return rc;
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = 0.0;
            for (int pass = 0; pass < 2; ++pass) {   // CGS2
                if ((rc = dots(j + 1, w))) return rc;
                for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] += std::complex<double>(hcoef[i].x, hcoef[i].y);
                k_multiaxpy<<<grid1(n), 256, 0, st>>>(w, V, n, j + 1, coef, -1.0);
            }
            double hn = 0.0;
            if ((rc = norm_of(w, &hn))) return rc;
            H[(size_t)(j + 1) * m + j] = hn;
            if (hn > 0.0) k_scale_copy<<<grid1(n), 256, 0, st>>>(w, V + (size_t)(j + 1) * n, n, 1.0 / hn);
            // Givens rotations
            for (int i = 0; i < j; ++i) {
                const std::complex<double> a = H[(size_t)i * m + j], bq = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = std::conj(cs[i]) * a + std::conj(sn[i]) * bq;
                H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * bq;
            }
            const std::complex<double> a = H[(size_t)j * m + j], bq = H[(size_t)(j + 1) * m + j];
            const double den = std::sqrt(std::norm(a) + std::norm(bq));
            cs[j] = den > 0 ? a / den : 1.0;
            sn[j] = den > 0 ? bq / den : 0.0;
            H[(size_t)j * m + j] = den;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = std::conj(cs[j]) * g[j];
            if (std::abs(g[j + 1]) / bnorm <= 0.5 * tol || hn == 0.0) { ++j; break; }
        }
        // y = H^-1 g (upper triangular j x j); x += Z y
        std::vector<std::complex<double>> y(j);
        for (int i = j - 1; i >= 0; --i) {
            std::complex<double> t = g[i];
            for (int k = i + 1; k < j; ++k) t -= H[(size_t)i * m + k] * y[k];
            y[i] = t / H[(size_t)i * m + i];
        }
        for (int i = 0; i < j; ++i) hcoef[i] = make_double2(y[i].real(), y[i].imag());
        CUDA_TRY(cudaMemcpyAsync(coef, hcoef.data(), j * sizeof(double2), cudaMemcpyHostToDevice, st));
        double2 *Zb = Z;
        k_multiaxpy<<<grid1(n), 256, 0, st>>>(xx, Zb, n, j, coef, 1.0);
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaMemcpyAsync(fac->h_err, fac->d_solve_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (*fac->h_err)
        return fail(FDFD_ERR_TIMEOUT, "solve_gmres: a bounded wait of the cooperative substitutions ran out (the "
                                      "solution is not valid)");
    CUDA_TRY(cudaEventRecord(fac->ev[3], st));
    fac->stats.refine_iters = apps - 1;
    fac->stats.rel_residual = rel;
    if (!(rel <= tol))
        return fail(FDFD_ERR_NOT_CONVERGED, "solve_gmres: residual " + std::to_string(rel) + " above tolerance after " +
                                                std::to_string(apps) + " factor applications");
    return FDFD_OK;
}

extern "C" int fdfd_factor_coef_get(const fdfd_factor *fac, void *dst, void *stream) {
    if (!fac || !dst) return fail(FDFD_ERR_BAD_ARG, "factor_coef_get: NULL argument");
    if (!fac->coef_valid)
        return fail(FDFD_ERR_BAD_ARG, "factor_coef_get: no stored coefficients (a numeric factorization of an "
                                      "operator given by eps and the 1/s vectors comes first)");
    CUDA_TRY(cudaMemcpyAsync(dst, fac->d_coef, (size_t)5 * fac->n * 16, cudaMemcpyDeviceToDevice,
                             (cudaStream_t)stream));
    return FDFD_OK;
}

extern "C" int fdfd_factor_stats_get(const fdfd_factor *fac, fdfd_factor_stats *st) {
    if (!fac || !st) return fail(FDFD_ERR_BAD_ARG, "factor_stats: NULL argument");
    fdfd_factor *f = const_cast<fdfd_factor *>(fac);
    float ms = 0.f;
    if (f->numeric_done && cudaEventSynchronize(f->ev[1]) == cudaSuccess &&
        cudaEventElapsedTime(&ms, f->ev[0], f->ev[1]) == cudaSuccess)
        f->stats.factor_ms = ms;
    if (cudaEventQuery(f->ev[3]) == cudaSuccess && cudaEventElapsedTime(&ms, f->ev[2], f->ev[3]) == cudaSuccess)
        f->stats.solve_ms = ms;
    cudaGetLastError();
    int tiny = 0;
    if (f->numeric_done && cudaMemcpy(&tiny, f->d_tiny, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)
        f->stats.tiny_pivots = tiny;
    int tce = 0;
    if (f->d_tcerr && cudaMemcpy(&tce, f->d_tcerr, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)
        f->stats.tc_errors = tce;
    *st = f->stats;
    return FDFD_OK;
}

extern "C" void fdfd_factor_destroy(fdfd_factor *fac) { free_factor(fac); }
