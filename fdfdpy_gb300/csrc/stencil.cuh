// Device-side description of the PML-stretched 2D Maxwell operator and the
// FP64 routine that produces one row of its 5-point stencil.
//
// The arithmetic follows construct_A (fdfdpy/linalg.py:41-107) operation by
// operation, without FMA contraction (explicit _rn intrinsics), so the
// assembled values track the scipy products and sums of the reference:
//   Ez: A = (Sxf Dxf / mu0') (Sxb Dxb) + (Syf Dyf / mu0') (Syb Dyb)
//         + omega^2 diag(eps0' eps)                      (linalg.py:52-66)
//   Hz: A = (Sxf Dxf) Tx^-1 (Sxb Dxb) + (Syf Dyf) Ty^-1 (Syb Dyb)
//         + omega^2 mu0' I                               (linalg.py:69-93)
// with eps0' = EPSILON_0 L0, mu0' = MU_0 L0, Tx/Ty the grid-averaged
// permittivities (linalg.py:16-22, 73-78) and S.. = diag(1/s) (pml.py:64-75).
// Derivatives are periodic (fdfdpy/derivatives.py:22-32).
#pragma once

#include <cuda_runtime.h>

#include "fdfd_internal.h"

namespace fdfd {

struct OpDev {
    int Nx, Ny, pol, averaging;
    // rows per problem of a batch of stacked grids (explicit-stencil
    // operators only): rows [b Nxp, (b + 1) Nxp) wrap among themselves;
    // 0 = one problem
    int Nxp;
    double invdx, invdy;  // 1/dx, 1/dy with dx = xlen/Nx (linalg.py:25-33)
    double invmu;         // 1/(MU_0*L0)
    double eps0L;         // EPSILON_0*L0
    double w2;            // omega**2
    double w2mu;          // omega**2 * (MU_0*L0)
    double w2e0L;         // (omega**2 * EPSILON_0) * L0  (simulation.py:67)
    const double *eps;
    const double *eps_add;
    const double2 *diag_add;
    const double2 *isxf, *isxb, *isyf, *isyb;
    const double2 *stencil;  // explicit coefficients [5][n], or NULL
};

// Validates a public operator description and derives the device scalars.
int make_opdev(const fdfd_operator *op, OpDev *d);

__device__ __forceinline__ double2 c_mul_rn(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 c_scale_rn(double2 a, double s) {
    return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s));
}
__device__ __forceinline__ double2 c_add_rn(double2 a, double2 b) {
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 c_sub_rn(double2 a, double2 b) {
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}

// eps0' * eps_r at a cell.
__device__ __forceinline__ double eps_e(const OpDev &o, int i, int j) {
    return __dmul_rn(o.eps0L, o.eps[(size_t)i * o.Ny + j]);
}

// 1/eps_x at (i, j): eps_x = (E[i-1, j] + E[i, j]) / 2 (grid_average 'x').
__device__ __forceinline__ double inv_eps_x(const OpDev &o, int i, int j) {
    const int im = (i == 0) ? o.Nx - 1 : i - 1;
    const double e = o.averaging ? __dmul_rn(__dadd_rn(eps_e(o, im, j), eps_e(o, i, j)), 0.5)
                                 : eps_e(o, i, j);
    return __ddiv_rn(1.0, e);
}
__device__ __forceinline__ double inv_eps_y(const OpDev &o, int i, int j) {
    const int jm = (j == 0) ? o.Ny - 1 : j - 1;
    const double e = o.averaging ? __dmul_rn(__dadd_rn(eps_e(o, i, jm), eps_e(o, i, j)), 0.5)
                                 : eps_e(o, i, j);
    return __ddiv_rn(1.0, e);
}

// Row (i, j) of A: c[0] centre, c[1] (i-1, j), c[2] (i+1, j), c[3] (i, j-1),
// c[4] (i, j+1), all complex128.
__device__ inline void stencil_row(const OpDev &o, int i, int j, double2 c[5]) {
    const int Nx = o.Nx, Ny = o.Ny;
    if (o.stencil) {
        const size_t n = (size_t)Nx * Ny, k = (size_t)i * Ny + j;
#pragma unroll
        for (int d = 0; d < 5; ++d) c[d] = o.stencil[d * n + k];
        return;
    }
    const int ip = (i == Nx - 1) ? 0 : i + 1;
    const int jp = (j == Ny - 1) ? 0 : j + 1;
    const size_t k = (size_t)i * Ny + j;
    const double vx = o.invdx, vy = o.invdy;
    // Rows of Dxf' = Sxf Dxf (entries a_i * (+-1/dx)) and columns of
    // Dxb' = Sxb Dxb (entries b_i * (+-1/dx)).
    double2 fxp = c_scale_rn(o.isxf[i], vx), fxn = c_scale_rn(o.isxf[i], -vx);
    double2 fyp = c_scale_rn(o.isyf[j], vy), fyn = c_scale_rn(o.isyf[j], -vy);
    const double2 bx0p = c_scale_rn(o.isxb[i], vx), bx0n = c_scale_rn(o.isxb[i], -vx);
    const double2 bx1n = c_scale_rn(o.isxb[ip], -vx), bx1p = c_scale_rn(o.isxb[ip], vx);
    const double2 by0p = c_scale_rn(o.isyb[j], vy), by0n = c_scale_rn(o.isyb[j], -vy);
    const double2 by1n = c_scale_rn(o.isyb[jp], -vy), by1p = c_scale_rn(o.isyb[jp], vy);
    double2 cx, cy, centre_add;
    if (o.pol == FDFD_POL_EZ) {
        // (Dxf * 1 / MU_0_) is a multiplication by the Python float 1/MU_0_.
        fxp = c_scale_rn(fxp, o.invmu); fxn = c_scale_rn(fxn, o.invmu);
        fyp = c_scale_rn(fyp, o.invmu); fyn = c_scale_rn(fyn, o.invmu);
        c[1] = c_mul_rn(fxn, bx0n);
        c[2] = c_mul_rn(fxp, bx1p);
        c[3] = c_mul_rn(fyn, by0n);
        c[4] = c_mul_rn(fyp, by1p);
        cx = c_add_rn(c_mul_rn(fxn, bx0p), c_mul_rn(fxp, bx1n));
        cy = c_add_rn(c_mul_rn(fyn, by0p), c_mul_rn(fyp, by1n));
        centre_add = make_double2(__dmul_rn(o.w2, __dmul_rn(o.eps0L, o.eps[k])), 0.0);
    } else {
        const double tx0 = inv_eps_x(o, i, j), tx1 = inv_eps_x(o, ip, j);
        const double ty0 = inv_eps_y(o, i, j), ty1 = inv_eps_y(o, i, jp);
        const double2 gxn = c_scale_rn(fxn, tx0), gxp = c_scale_rn(fxp, tx1);
        const double2 gyn = c_scale_rn(fyn, ty0), gyp = c_scale_rn(fyp, ty1);
        c[1] = c_mul_rn(gxn, bx0n);
        c[2] = c_mul_rn(gxp, bx1p);
        c[3] = c_mul_rn(gyn, by0n);
        c[4] = c_mul_rn(gyp, by1p);
        cx = c_add_rn(c_mul_rn(gxn, bx0p), c_mul_rn(gxp, bx1n));
        cy = c_add_rn(c_mul_rn(gyn, by0p), c_mul_rn(gyp, by1n));
        centre_add = make_double2(o.w2mu, 0.0);
    }
    double2 ctr = c_add_rn(c_add_rn(cx, cy), centre_add);
    if (o.eps_add) ctr.x = __dadd_rn(ctr.x, __dmul_rn(o.w2e0L, o.eps_add[k]));
    if (o.diag_add) ctr = c_add_rn(ctr, o.diag_add[k]);
    c[0] = ctr;
}

// Neighbour cell index in direction d (0 xm, 1 xp, 2 ym, 3 yp) and the
// direction that points back.
__device__ __forceinline__ int nbr_cell(const OpDev &o, int i, int j, int d) {
    if (o.Nxp && d < 2) {
        const int i0 = i - i % o.Nxp;
        if (d == 0) return ((i == i0) ? i0 + o.Nxp - 1 : i - 1) * o.Ny + j;
        return ((i == i0 + o.Nxp - 1) ? i0 : i + 1) * o.Ny + j;
    }
    switch (d) {
        case 0: return ((i == 0) ? o.Nx - 1 : i - 1) * o.Ny + j;
        case 1: return ((i == o.Nx - 1) ? 0 : i + 1) * o.Ny + j;
        case 2: return i * o.Ny + ((j == 0) ? o.Ny - 1 : j - 1);
        default: return i * o.Ny + ((j == o.Ny - 1) ? 0 : j + 1);
    }
}
__device__ __forceinline__ int opposite_dir(int d) { return d ^ 1; }

}  // namespace fdfd
