// Stencil kernels of the FDFD engine: PML stretch factors, CSR assembly
// (K1), derivative operators, the matrix-free FP64 residual (K2), field
// recovery (K8), the adjoint gradient (K9) and column norms.
//
// All of these are HBM-bound elementwise/stencil passes: one thread per
// cell, consecutive threads on consecutive j (the contiguous axis of the C
// order k = i*Ny + j), 256-thread blocks, grids sized in multiples of the
// SM count by the grid-stride loops.
#include <cuda_runtime.h>

#include <cmath>

#include "stencil.cuh"

namespace fdfd {

namespace {

constexpr int kThreads = 256;

inline int grid_for(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;  // grid-stride beyond 32 blocks per SM
    return (int)b;
}

// ---- PML ----------------------------------------------------------------
// 1/s with numpy's complex division (Smith's algorithm, as numpy's complex
// true_divide implements it) so that 1/s_vector in S_create
// (fdfdpy/pml.py:69-75) is reproduced.
__device__ double2 recip_smith(double2 s) {
    const double ar = fabs(s.x), ai = fabs(s.y);
    if (ar >= ai) {
        const double rat = __ddiv_rn(s.y, s.x);
        const double scl = __ddiv_rn(1.0, __dadd_rn(s.x, __dmul_rn(s.y, rat)));
        return make_double2(__dmul_rn(1.0, scl), __dmul_rn(__dsub_rn(0.0, rat), scl));
    } else {
        const double rat = __ddiv_rn(s.x, s.y);
        const double scl = __ddiv_rn(1.0, __dadd_rn(s.y, __dmul_rn(s.x, rat)));
        return make_double2(__dmul_rn(rat, scl), __dmul_rn(-1.0, scl));
    }
}

// x**4 to within about half an ulp: x^2 as an exact double-double (Dekker's
// two-product through fma), then squared.
__device__ double pow4(double x) {
    const double x2 = __dmul_rn(x, x);
    const double e2 = fma(x, x, -x2);
    const double hi = __dmul_rn(x2, x2);
    const double lo = fma(x2, x2, -hi) + 2.0 * x2 * e2;
    return hi + lo;
}

// create_sfactor (fdfdpy/pml.py:20-39) for the 'f' and 'b' grids of one
// axis, followed by the reciprocal taken in S_create (pml.py:69-75).
//   sig_w (pml.py:7-11): sig_max (l/dw)^4, sig_max = 60 / ((2 eta0) dw)
//   S     (pml.py:14-17): 1 - 1j sig / (omega eps0 L0)
__global__ void k_sfactors(int Nw, int Npml, double hw, double dw, double sig_max,
                           double inv_den, double2 *inv_f, double2 *inv_b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Nw; i += gridDim.x * blockDim.x) {
        double2 sf = make_double2(1.0, 0.0), sb = make_double2(1.0, 0.0);
        if (Npml >= 1) {
            double lf = -1.0, lb = -1.0;
            if (i <= Npml) {
                lf = __dmul_rn(hw, (double)(Npml - i) + 0.5);
                lb = __dmul_rn(hw, (double)(Npml - i + 1));
            } else if (i > Nw - Npml) {
                lf = __dmul_rn(hw, (double)(i - (Nw - Npml)) - 0.5);
                lb = __dmul_rn(hw, (double)(i - (Nw - Npml) - 1));
            }
            if (lf >= 0.0) {
                const double sig = __dmul_rn(sig_max, pow4(__ddiv_rn(lf, dw)));
                sf = make_double2(1.0, -__dmul_rn(sig, inv_den));
            }
            if (lb >= 0.0) {
                const double sig = __dmul_rn(sig_max, pow4(__ddiv_rn(lb, dw)));
                sb = make_double2(1.0, -__dmul_rn(sig, inv_den));
            }
        }
        inv_f[i] = recip_smith(sf);
        inv_b[i] = recip_smith(sb);
    }
}

// ---- K1: CSR assembly ---------------------------------------------------
__global__ void k_assemble_csr(OpDev o, int32_t *indptr, int32_t *indices, double2 *data) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / o.Ny), j = (int)(k % o.Ny);
        double2 c[5];
        stencil_row(o, i, j, c);
        int col[5] = {(int)k, nbr_cell(o, i, j, 0), nbr_cell(o, i, j, 1), nbr_cell(o, i, j, 2),
                      nbr_cell(o, i, j, 3)};
        // Insertion sort of 5 (column, value) pairs: canonical CSR order.
        for (int a = 1; a < 5; ++a) {
            const int cc = col[a];
            const double2 vv = c[a];
            int b = a - 1;
            while (b >= 0 && col[b] > cc) {
                col[b + 1] = col[b];
                c[b + 1] = c[b];
                --b;
            }
            col[b + 1] = cc;
            c[b + 1] = vv;
        }
        indptr[k] = (int32_t)(5 * k);
        for (int a = 0; a < 5; ++a) {
            indices[5 * k + a] = col[a];
            data[5 * k + a] = c[a];
        }
        if (k == n - 1) indptr[n] = (int32_t)(5 * n);
    }
}

// One derivative operator with its S factor (fdfdpy/linalg.py:59-62,
// 86-89): which 0 Dxf, 1 Dxb, 2 Dyf, 3 Dyb; 2 entries per row.
__global__ void k_deriv_csr(OpDev o, int which, int32_t *indptr, int32_t *indices, double2 *data) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / o.Ny), j = (int)(k % o.Ny);
        int c0 = (int)k, c1;
        double2 v0, v1;
        switch (which) {
            case 0:  // forward x: -1 on the diagonal, +1 at (i+1)
                v0 = c_scale_rn(o.isxf[i], -o.invdx);
                v1 = c_scale_rn(o.isxf[i], o.invdx);
                c1 = nbr_cell(o, i, j, 1);
                break;
            case 1:  // backward x: +1 on the diagonal, -1 at (i-1)
                v0 = c_scale_rn(o.isxb[i], o.invdx);
                v1 = c_scale_rn(o.isxb[i], -o.invdx);
                c1 = nbr_cell(o, i, j, 0);
                break;
            case 2:
                v0 = c_scale_rn(o.isyf[j], -o.invdy);
                v1 = c_scale_rn(o.isyf[j], o.invdy);
                c1 = nbr_cell(o, i, j, 3);
                break;
            default:
                v0 = c_scale_rn(o.isyb[j], o.invdy);
                v1 = c_scale_rn(o.isyb[j], -o.invdy);
                c1 = nbr_cell(o, i, j, 2);
                break;
        }
        indptr[k] = (int32_t)(2 * k);
        if (c1 < c0) {
            indices[2 * k] = c1; data[2 * k] = v1;
            indices[2 * k + 1] = c0; data[2 * k + 1] = v0;
        } else {
            indices[2 * k] = c0; data[2 * k] = v0;
            indices[2 * k + 1] = c1; data[2 * k + 1] = v1;
        }
        if (k == n - 1) indptr[n] = (int32_t)(2 * n);
    }
}

__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
    return acc;
}

// ---- K2: matrix-free residual / apply -----------------------------------
// mode 0: r = b - A x;  1: y = A x;  2: y = A^T x;  3: r = b - A^T x.
__global__ void k_apply(OpDev o, const double2 *__restrict__ x, const double2 *__restrict__ b,
                        double2 *__restrict__ out, int nrhs, int mode) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    const bool transpose = (mode == 2 || mode == 3);
    const bool residual = (mode == 0 || mode == 3);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / o.Ny), j = (int)(k % o.Ny);
        double2 c[5];
        int nb[4];
        for (int d = 0; d < 4; ++d) nb[d] = nbr_cell(o, i, j, d);
        if (!transpose) {
            stencil_row(o, i, j, c);
        } else {
            // Column k of A: A[k,k] and A[t,k] for each neighbour t.
            double2 ct[5];
            stencil_row(o, i, j, ct);
            c[0] = ct[0];
            for (int d = 0; d < 4; ++d) {
                const int t = nb[d];
                stencil_row(o, t / o.Ny, t % o.Ny, ct);
                c[1 + d] = ct[1 + opposite_dir(d)];
            }
        }
        for (int r = 0; r < nrhs; ++r) {
            const double2 *xr = x + (size_t)r * n;
            double2 acc = make_double2(0.0, 0.0);
            acc = cfma(c[0], xr[k], acc);
            for (int d = 0; d < 4; ++d) acc = cfma(c[1 + d], xr[nb[d]], acc);
            if (residual) {
                const double2 bb = b[(size_t)r * n + k];
                out[(size_t)r * n + k] = make_double2(bb.x - acc.x, bb.y - acc.y);
            } else {
                out[(size_t)r * n + k] = acc;
            }
        }
    }
}

// ---- K8: field recovery (fdfdpy/simulation.py:129-175) -------------------
// Ez: f1 = s1 * (Dyb' X), f2 = s2 * (Dxb' X)
// Hz: f1 = s1 * (Ty^-1 Dyb' X), f2 = s2 * (Tx^-1 Dxb' X)
__global__ void k_fields(OpDev o, const double2 *__restrict__ X, double2 *__restrict__ f1,
                         double2 *__restrict__ f2, double2 s1, double2 s2) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / o.Ny), j = (int)(k % o.Ny);
        double2 dyd = c_scale_rn(o.isyb[j], o.invdy), dyo = c_scale_rn(o.isyb[j], -o.invdy);
        double2 dxd = c_scale_rn(o.isxb[i], o.invdx), dxo = c_scale_rn(o.isxb[i], -o.invdx);
        if (o.pol == FDFD_POL_HZ) {
            const double ty = inv_eps_y(o, i, j), tx = inv_eps_x(o, i, j);
            dyd = c_scale_rn(dyd, ty); dyo = c_scale_rn(dyo, ty);
            dxd = c_scale_rn(dxd, tx); dxo = c_scale_rn(dxo, tx);
        }
        const double2 xk = X[k];
        const double2 gy = c_add_rn(c_mul_rn(dyd, xk), c_mul_rn(dyo, X[nbr_cell(o, i, j, 2)]));
        const double2 gx = c_add_rn(c_mul_rn(dxd, xk), c_mul_rn(dxo, X[nbr_cell(o, i, j, 0)]));
        f1[k] = c_mul_rn(s1, gy);
        f2[k] = c_mul_rn(s2, gx);
    }
}

// ---- mode-source slice operator (fdfdpy/source/mode.py:76-91) ------------
__global__ void k_mode_stencil(int N, int pol, int average, const double *eps, double w2mu0,
                               double eps0L, double v, double shift, double2 *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const int im = (i == 0) ? N - 1 : i - 1, ip = (i == N - 1) ? 0 : i + 1;
        const double e = __dmul_rn(eps0L, eps[i]);
        double c, xm, xp;
        // Dxf Dxb rows: (-v)(v e_i - v e_{i-1}) + v (v e_{i+1} - v e_i)
        const double vv = __dmul_rn(v, v);
        if (pol == FDFD_POL_EZ) {
            xm = vv;
            xp = vv;
            c = __dadd_rn(__dmul_rn(w2mu0, e), __dsub_rn(-vv, vv));
        } else {
            // eps_x = eps0' * grid_average(eps): averaged along the slice
            // only when the slice runs along the rolled axis
            const double ax0 = average ? __dmul_rn(__dadd_rn(eps[im], eps[i]), 0.5) : eps[i];
            const double ax1 = average ? __dmul_rn(__dadd_rn(eps[i], eps[ip]), 0.5) : eps[ip];
            const double t0 = __ddiv_rn(1.0, __dmul_rn(eps0L, ax0));
            const double t1 = __ddiv_rn(1.0, __dmul_rn(eps0L, ax1));
            // ((T_eps Dxf) T_epsx^-1) Dxb, evaluated left to right
            const double ev = __dmul_rn(e, v);
            xm = __dmul_rn(__dmul_rn(ev, t0), v);
            xp = __dmul_rn(__dmul_rn(ev, t1), v);
            c = __dadd_rn(__dmul_rn(w2mu0, e), -__dadd_rn(xm, xp));
        }
        out[i] = make_double2(c - shift, 0.0);
        out[N + i] = make_double2(xm, 0.0);
        out[2 * N + i] = make_double2(xp, 0.0);
        out[3 * N + i] = make_double2(0.0, 0.0);
        out[4 * N + i] = make_double2(0.0, 0.0);
    }
}

// ---- K9: adjoint gradient ------------------------------------------------
__global__ void k_grad_eps(int64_t n, double coef, const double2 *__restrict__ lam,
                           const double2 *__restrict__ E, double *__restrict__ g) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = lam[k], e = E[k];
        g[k] = coef * (a.x * e.x - a.y * e.y);
    }
}

// K9 for Hz.  A = Dxf' Tx^-1 Dxb' + Dyf' Ty^-1 Dyb' + omega^2 mu0' I with
// Tx = diag(eps_x), eps_x = eps0' (eps[i-1, j] + eps[i, j]) / 2 (or eps0' eps
// without averaging; linalg.py:69-93).  With u = Dxf'^T lambda and
// v = Dxb' X:  lambda^T (dA / d eps_x[q]) X = -u_q v_q / eps_x[q]^2, so
//   dL/d eps_r[p] = sum_{q : eps_x[q] depends on eps_r[p]}
//                   (d eps_x[q] / d eps_r[p]) Re(u_q v_q) / eps_x[q]^2  (+ y)
// where q ranges over p and its +x (+y) neighbour with averaging (weight
// eps0'/2 each), over p alone without (weight eps0').
__device__ __forceinline__ double hz_term_x(const OpDev &o, const double2 *lam, const double2 *X, int i, int j) {
    const int im = (i == 0) ? o.Nx - 1 : i - 1;
    const size_t k = (size_t)i * o.Ny + j, km = (size_t)im * o.Ny + j;
    // u = Dxf'^T lambda at (i, j): column (i, j) of Sxf Dxf
    const double2 a = c_mul_rn(o.isxf[im], lam[km]), b = c_mul_rn(o.isxf[i], lam[k]);
    const double2 u = c_scale_rn(c_sub_rn(a, b), o.invdx);
    const double2 v = c_scale_rn(c_mul_rn(o.isxb[i], c_sub_rn(X[k], X[km])), o.invdx);
    const double t = inv_eps_x(o, i, j);
    return (u.x * v.x - u.y * v.y) * t * t;
}
__device__ __forceinline__ double hz_term_y(const OpDev &o, const double2 *lam, const double2 *X, int i, int j) {
    const int jm = (j == 0) ? o.Ny - 1 : j - 1;
    const size_t k = (size_t)i * o.Ny + j, km = (size_t)i * o.Ny + jm;
    const double2 a = c_mul_rn(o.isyf[jm], lam[km]), b = c_mul_rn(o.isyf[j], lam[k]);
    const double2 u = c_scale_rn(c_sub_rn(a, b), o.invdy);
    const double2 v = c_scale_rn(c_mul_rn(o.isyb[j], c_sub_rn(X[k], X[km])), o.invdy);
    const double t = inv_eps_y(o, i, j);
    return (u.x * v.x - u.y * v.y) * t * t;
}

__global__ void k_grad_eps_hz(OpDev o, const double2 *__restrict__ lam, const double2 *__restrict__ X,
                              double *__restrict__ g) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / o.Ny), j = (int)(k % o.Ny);
        double s = hz_term_x(o, lam, X, i, j) + hz_term_y(o, lam, X, i, j);
        if (o.averaging) {
            const int ip = (i == o.Nx - 1) ? 0 : i + 1, jp = (j == o.Ny - 1) ? 0 : j + 1;
            s += hz_term_x(o, lam, X, ip, j) + hz_term_y(o, lam, X, i, jp);
            s *= 0.5;
        }
        g[k] = o.eps0L * s;
    }
}

// ---- norms ----------------------------------------------------------------
__global__ void k_sumsq_partial(const double2 *__restrict__ v, int64_t n, double *partial) {
    __shared__ double red[kThreads / 32];
    const int col = blockIdx.y;
    const double2 *vc = v + (size_t)col * n;
    double s = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = vc[k];
        s = fma(a.x, a.x, s);
        s = fma(a.y, a.y, s);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) partial[(size_t)col * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void k_sumsq_final(const double *partial, int nparts, double *out) {
    __shared__ double red[kThreads / 32];
    const int col = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += partial[(size_t)col * nparts + b];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) out[col] = sqrt(s);
    }
}

}  // namespace

// ---- host helpers shared with the factor --------------------------------
constexpr int kNormParts = 152 * 4;

int norms_device(const void *v, int64_t n, int ncol, double *partial, double *out_dev,
                 cudaStream_t st) {
    k_sumsq_partial<<<dim3(kNormParts, ncol), kThreads, 0, st>>>((const double2 *)v, n, partial);
    k_sumsq_final<<<ncol, kThreads, 0, st>>>(partial, kNormParts, out_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string("norms: ") + cudaGetErrorString(e));
    return FDFD_OK;
}
size_t norms_partial_count(int ncol) { return (size_t)kNormParts * ncol; }

int apply_device(const OpDev &o, const void *x, const void *b, void *out, int nrhs, int mode,
                 cudaStream_t st) {
    const int64_t n = (int64_t)o.Nx * o.Ny;
    k_apply<<<grid_for(n), kThreads, 0, st>>>(o, (const double2 *)x, (const double2 *)b,
                                              (double2 *)out, nrhs, mode);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string("apply: ") + cudaGetErrorString(e));
    return FDFD_OK;
}

int make_opdev(const fdfd_operator *op, OpDev *d) {
    if (!op) return fail(FDFD_ERR_BAD_ARG, "operator is NULL");
    if (op->stencil) {
        if (op->Nx < 1 || op->Ny < 1) return fail(FDFD_ERR_BAD_ARG, "operator: empty grid");
    } else if (op->Nx < 3 || op->Ny < 3) {
        return fail(FDFD_ERR_BAD_ARG, "operator: the GPU operator needs Nx >= 3 and Ny >= 3");
    }
    if ((int64_t)op->Nx * op->Ny > ((int64_t)1 << 30) / 5)
        return fail(FDFD_ERR_BAD_ARG, "operator: grid too large for int32 CSR indices");
    if (op->pol != FDFD_POL_EZ && op->pol != FDFD_POL_HZ)
        return fail(FDFD_ERR_BAD_ARG, "operator: pol must be FDFD_POL_EZ or FDFD_POL_HZ");
    if (!op->stencil && (!op->eps || !op->inv_sxf || !op->inv_sxb || !op->inv_syf || !op->inv_syb))
        return fail(FDFD_ERR_BAD_ARG, "operator: eps and the four 1/s vectors are required");
    if (!op->stencil && (!(op->xlen > 0.0) || !(op->ylen > 0.0) || !(op->L0 > 0.0)))
        return fail(FDFD_ERR_BAD_ARG, "operator: xlen, ylen and L0 must be positive");
    d->stencil = (const double2 *)op->stencil;
    d->Nxp = 0;
    if (op->stencil) {
        d->Nx = op->Nx; d->Ny = op->Ny; d->pol = op->pol; d->averaging = 0;
        d->invdx = d->invdy = d->invmu = d->eps0L = d->w2 = d->w2mu = d->w2e0L = 0.0;
        d->eps = nullptr; d->eps_add = nullptr; d->diag_add = nullptr;
        d->isxf = (const double2 *)op->inv_sxf; d->isxb = (const double2 *)op->inv_sxb;
        d->isyf = (const double2 *)op->inv_syf; d->isyb = (const double2 *)op->inv_syb;
        return FDFD_OK;
    }
    d->Nx = op->Nx; d->Ny = op->Ny; d->pol = op->pol; d->averaging = op->averaging ? 1 : 0;
    const double dx = op->xlen / op->Nx, dy = op->ylen / op->Ny;  // linalg.py:25-33
    d->invdx = 1.0 / dx;
    d->invdy = 1.0 / dy;
    const double mu0L = MU_0 * op->L0;
    d->invmu = 1.0 / mu0L;
    d->eps0L = EPSILON_0 * op->L0;
    d->w2 = op->omega * op->omega;
    d->w2mu = d->w2 * mu0L;
    d->w2e0L = (d->w2 * EPSILON_0) * op->L0;
    d->eps = op->eps;
    d->eps_add = op->eps_add;
    d->diag_add = (const double2 *)op->diag_add;
    d->isxf = (const double2 *)op->inv_sxf;
    d->isxb = (const double2 *)op->inv_sxb;
    d->isyf = (const double2 *)op->inv_syf;
    d->isyb = (const double2 *)op->inv_syb;
    return FDFD_OK;
}

}  // namespace fdfd

// ---- C ABI ----------------------------------------------------------------
using namespace fdfd;

static int launch_status(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return FDFD_OK;
}

extern "C" int fdfd_pml_sfactors(int32_t Nw, int32_t Nw_pml, double wlen, double omega, double L0,
                                 void *out_inv_f, void *out_inv_b, void *stream) {
    if (Nw < 1 || !out_inv_f || !out_inv_b) return fail(FDFD_ERR_BAD_ARG, "pml_sfactors: bad size or NULL output");
    if (!(omega > 0.0) || !(L0 > 0.0) || !(wlen > 0.0))
        return fail(FDFD_ERR_BAD_ARG, "pml_sfactors: omega, L0 and wlen must be positive");
    const double hw = wlen / Nw;                          // pml.py:27
    const double dw = (double)Nw_pml * hw;                // pml.py:28
    const double eta0 = std::sqrt(MU_0 / EPSILON_0);      // constants.py:6
    const double sig_max = 60.0 / ((2.0 * eta0) * dw);    // pml.py:10, -(m+1) lnR = 60
    const double inv_den = 1.0 / ((omega * EPSILON_0) * L0);  // pml.py:17
    k_sfactors<<<grid_for(Nw), kThreads, 0, (cudaStream_t)stream>>>(
        Nw, Nw_pml, hw, dw, sig_max, inv_den, (double2 *)out_inv_f, (double2 *)out_inv_b);
    return launch_status("pml_sfactors");
}

extern "C" int fdfd_assemble_csr(const fdfd_operator *op, int32_t *indptr, int32_t *indices,
                                 void *data, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (o.stencil) return fail(FDFD_ERR_BAD_ARG, "assemble_csr: needs the physical operator, not a stencil");
    if (!indptr || !indices || !data) return fail(FDFD_ERR_BAD_ARG, "assemble_csr: NULL output");
    const int64_t n = (int64_t)o.Nx * o.Ny;
    k_assemble_csr<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(o, indptr, indices,
                                                                      (double2 *)data);
    return launch_status("assemble_csr");
}

extern "C" int fdfd_assemble_deriv_csr(const fdfd_operator *op, int32_t which, int32_t *indptr,
                                       int32_t *indices, void *data, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (o.stencil) return fail(FDFD_ERR_BAD_ARG, "assemble_deriv_csr: needs the physical operator, not a stencil");
    if (which < 0 || which > 3) return fail(FDFD_ERR_BAD_ARG, "assemble_deriv_csr: which must be 0..3");
    if (!indptr || !indices || !data) return fail(FDFD_ERR_BAD_ARG, "assemble_deriv_csr: NULL output");
    const int64_t n = (int64_t)o.Nx * o.Ny;
    k_deriv_csr<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(o, which, indptr, indices,
                                                                   (double2 *)data);
    return launch_status("assemble_deriv_csr");
}

extern "C" int fdfd_residual(const fdfd_operator *op, const void *x, const void *b, void *r,
                             int32_t nrhs, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (!x || !b || !r || nrhs < 1) return fail(FDFD_ERR_BAD_ARG, "residual: NULL buffer or nrhs < 1");
    return apply_device(o, x, b, r, nrhs, 0, (cudaStream_t)stream);
}

extern "C" int fdfd_apply(const fdfd_operator *op, const void *x, void *y, int32_t nrhs,
                          int32_t transpose, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (!x || !y || nrhs < 1) return fail(FDFD_ERR_BAD_ARG, "apply: NULL buffer or nrhs < 1");
    return apply_device(o, x, nullptr, y, nrhs, transpose ? 2 : 1, (cudaStream_t)stream);
}

extern "C" int fdfd_fields(const fdfd_operator *op, const void *X, void *f1, void *f2, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (o.stencil) return fail(FDFD_ERR_BAD_ARG, "fields: needs the physical operator, not a stencil");
    if (!X || !f1 || !f2) return fail(FDFD_ERR_BAD_ARG, "fields: NULL buffer");
    // Scalars of fdfdpy/simulation.py:148-149 (Hz) and 163-164 (Ez), as
    // Python evaluates them: -1/1j = 1j, 1/1j = -1j, then divisions by
    // omega (and mu0') of the imaginary part.
    const double inv_w = 1.0 / op->omega;
    double2 s1, s2;
    if (o.pol == FDFD_POL_EZ) {
        const double mu0L = MU_0 * op->L0;
        s1 = make_double2(0.0, inv_w / mu0L);       // -1/1j/omega/MU_0_
        s2 = make_double2(0.0, (-inv_w) / mu0L);    //  1/1j/omega/MU_0_
    } else {
        s1 = make_double2(0.0, -inv_w);             //  1/1j/omega
        s2 = make_double2(0.0, inv_w);              // -1/1j/omega
    }
    const int64_t n = (int64_t)o.Nx * o.Ny;
    k_fields<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(o, (const double2 *)X, (double2 *)f1,
                                                                (double2 *)f2, s1, s2);
    return launch_status("fields");
}

extern "C" int fdfd_adjoint_grad_eps(const fdfd_operator *op, const void *lambda_, const void *E,
                                     double *grad, void *stream) {
    OpDev o;
    int st = make_opdev(op, &o);
    if (st) return st;
    if (o.stencil) return fail(FDFD_ERR_BAD_ARG, "adjoint_grad_eps: needs the physical operator, not a stencil");
    if (!lambda_ || !E || !grad) return fail(FDFD_ERR_BAD_ARG, "adjoint_grad_eps: NULL buffer");
    const int64_t n = (int64_t)o.Nx * o.Ny;
    if (o.pol == FDFD_POL_HZ) {
        k_grad_eps_hz<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(o, (const double2 *)lambda_,
                                                                         (const double2 *)E, grad);
        return launch_status("adjoint_grad_eps");
    }
    const double coef = -(o.w2 * o.eps0L);
    k_grad_eps<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(n, coef, (const double2 *)lambda_,
                                                                  (const double2 *)E, grad);
    return launch_status("adjoint_grad_eps");
}

extern "C" int fdfd_norms(const void *v, int64_t n, int32_t ncol, double *out_host, void *stream) {
    if (!v || !out_host || n < 1 || ncol < 1) return fail(FDFD_ERR_BAD_ARG, "norms: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    double *buf = nullptr;
    const size_t parts = norms_partial_count(ncol);
    cudaError_t e = cudaMallocAsync((void **)&buf, (parts + ncol) * sizeof(double), st);
    if (e != cudaSuccess) return fail(FDFD_ERR_OOM, std::string("norms: ") + cudaGetErrorString(e));
    int rc = norms_device(v, n, ncol, buf, buf + parts, st);
    if (rc == FDFD_OK) {
        e = cudaMemcpyAsync(out_host, buf + parts, ncol * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = fail(FDFD_ERR_CUDA, std::string("norms: ") + cudaGetErrorString(e));
    }
    cudaFreeAsync(buf, st);
    return rc;
}

extern "C" int fdfd_mode_stencil(int32_t N, int32_t pol, int32_t average, const double *eps_slice,
                                 double omega, double dl, double L0, double shift, void *out,
                                 void *stream) {
    if (N < 1 || !eps_slice || !out) return fail(FDFD_ERR_BAD_ARG, "mode_stencil: bad size or NULL buffer");
    if (pol != FDFD_POL_EZ && pol != FDFD_POL_HZ) return fail(FDFD_ERR_BAD_ARG, "mode_stencil: bad pol");
    if (!(dl > 0.0) || !(L0 > 0.0)) return fail(FDFD_ERR_BAD_ARG, "mode_stencil: dl and L0 must be positive");
    const double w2mu0 = (omega * omega) * (MU_0 * L0);  // np.square(omega)*MU_0_
    const double v = 1.0 / dl;
    k_mode_stencil<<<grid_for(N), kThreads, 0, (cudaStream_t)stream>>>(N, pol, average, eps_slice, w2mu0,
                                                                      EPSILON_0 * L0, v, shift,
                                                                      (double2 *)out);
    return launch_status("mode_stencil");
}

// ---- column norms without any device allocation -----------------------------
// Some callers cannot allocate device memory at call time: a process whose
// device memory is fully reserved by its own allocator (a serving loop with
// a fixed budget, a framework's caching allocator holding the rest of HBM)
// would see cudaMallocAsync fail or stall on allocator synchronisation in
// the middle of an optimisation loop.  fdfd_norms_noalloc serves them from a
// fixed scratch array in the library's static device memory instead; every
// GPU that loads the library holds that array until the process exits.
namespace {
constexpr int kNoAllocMaxCols = 8;  // columns per call (documented limit)
constexpr size_t kNoAllocDoubles = (size_t)kNormParts * kNoAllocMaxCols + kNoAllocMaxCols;
static __device__ __align__(256) double g_norms_scratch[kNoAllocDoubles];

// Device address of the scratch array in the current context (host code
// may not take the address of a __device__ symbol directly: the host-side
// name is only a stand-in).  Looked up on every call -- a cheap query, and
// a cached address would go stale once the context is reset and the module
// loaded again.
int noalloc_scratch(double **out) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_norms_scratch);
    if (e != cudaSuccess || !ptr)
        return fail(e == cudaErrorNoDevice ? FDFD_ERR_NO_DEVICE : FDFD_ERR_CUDA,
                    std::string("norms_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    *out = (double *)ptr;
    return FDFD_OK;
}
}  // namespace

extern "C" int fdfd_norms_noalloc(const void *v, int64_t n, int32_t ncol, double *out_host, void *stream) {
    if (!v || !out_host || n < 1 || ncol < 1) return fail(FDFD_ERR_BAD_ARG, "norms_noalloc: bad argument");
    if (ncol > kNoAllocMaxCols)
        return fail(FDFD_ERR_BAD_ARG, "norms_noalloc: at most " + std::to_string(kNoAllocMaxCols) +
                                          " columns per call (fixed scratch); got " + std::to_string(ncol));
    double *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // Every partial-sum slot read by the final reduction is written by the
    // first kernel of this same call, so nothing has to be cleared first.
    double *partial = scratch, *out_dev = scratch + (size_t)kNormParts * kNoAllocMaxCols;
    rc = norms_device(v, n, ncol, partial, out_dev, st);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(out_host, out_dev, ncol * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string("norms_noalloc: ") + cudaGetErrorString(e));
    return FDFD_OK;
}
