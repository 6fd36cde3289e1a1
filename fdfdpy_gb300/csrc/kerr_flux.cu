// Kerr terms of the nonlinear solves (K1-NL) and the flux-probe reduction.
//
// K1-NL evaluates, in one pass over the grid, what fdfdpy computes with
// numpy expressions in three places: the Kerr permittivity and its
// derivatives (fdfdpy/nonlinearity.py:18-34), their sum over the
// nonlinearities (Simulation.compute_nl, fdfdpy/simulation.py:57-68) and
// the field-dependent terms of the Newton Jacobian
// (fdfdpy/nonlinear_solvers.py:117-149):
//   s        = (eps_r - 1) / (eps_max - 1)  with eps_scale, else 1
//   eps_nl   = 3 chi region |E|^2 s
//   dnl_deps = 3 chi region |E|^2 / (eps_max - 1)  with eps_scale, else 0
//   dnl_de   = 3 chi region conj(E) s
//   dAde     = dnl_de * omega^2 eps0 L0
//   jac_diag = dAde * E        (added to the diagonal of J11)
//   jac_off  = conj(dAde) * E  (the diagonal of J12)
// HBM-bound: one thread per cell, 16 B of E, 16 B of eps_r and region in,
// up to 8 + 8 + 16 + 16 + 16 B out.
//
// The flux probe (fdfdpy/simulation.py:260-315) is a reduction over one
// line of cells: dl * coef * sum_t Re(avg(F)_t * conj(G_t)), with F the
// field the reference averages across the line (Ez for Ez, Hz for Hz) and G
// the transverse partner (Hy/Hx, Ey/Ex).  One CTA, a fixed summation tree
// (deterministic), result left on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "fdfd_internal.h"

namespace fdfd {
namespace {

constexpr int kThreads = 256;

inline int grid_for(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
}

__global__ void k_kerr_assemble(int64_t n, const double2 *__restrict__ E, const double *__restrict__ eps_r,
                                const double *__restrict__ region, double three_chi, int eps_scale,
                                double inv_epsm1, double w2e0L, int accumulate, double *__restrict__ eps_nl,
                                double *__restrict__ dnl_deps, double2 *__restrict__ dnl_de,
                                double2 *__restrict__ jac_diag, double2 *__restrict__ jac_off) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double2 e = E[k];
        const double a2 = e.x * e.x + e.y * e.y;
        const double cr = three_chi * region[k];
        const double s = eps_scale ? (eps_r[k] - 1.0) * inv_epsm1 : 1.0;
        const double enl = cr * a2 * s;
        // dAde = cr * s * w2e0L * conj(e); dAde * e is real, conj(dAde) * e = c e^2
        const double c = cr * s * w2e0L;
        const double2 jd = make_double2(c * a2, 0.0);
        const double2 jo = make_double2(c * (e.x * e.x - e.y * e.y), c * (2.0 * e.x * e.y));
        const double2 de = make_double2(cr * s * e.x, -(cr * s * e.y));
        if (accumulate) {
            if (dnl_de) { double2 t = dnl_de[k]; dnl_de[k] = make_double2(t.x + de.x, t.y + de.y); }
            if (eps_nl) eps_nl[k] += enl;
            if (dnl_deps) dnl_deps[k] += eps_scale ? cr * a2 * inv_epsm1 : 0.0;
            if (jac_diag) { double2 t = jac_diag[k]; jac_diag[k] = make_double2(t.x + jd.x, t.y + jd.y); }
            if (jac_off) { double2 t = jac_off[k]; jac_off[k] = make_double2(t.x + jo.x, t.y + jo.y); }
        } else {
            if (eps_nl) eps_nl[k] = enl;
            if (dnl_deps) dnl_deps[k] = eps_scale ? cr * a2 * inv_epsm1 : 0.0;
            if (dnl_de) dnl_de[k] = de;
            if (jac_diag) jac_diag[k] = jd;
            if (jac_off) jac_off[k] = jo;
        }
    }
}

// sum_t Re(((F[k_t] + F[k_t + avg]) / 2) * conj(G[k_t])), k_t = base + t * step
__global__ void __launch_bounds__(kThreads) k_flux_line(const double2 *__restrict__ F,
                                                         const double2 *__restrict__ G, int64_t base,
                                                         int64_t step, int64_t avg, int len, double scale,
                                                         double *out) {
    __shared__ double red[kThreads / 32];
    double s = 0.0;
    for (int t = threadIdx.x; t < len; t += kThreads) {
        const int64_t k = base + (int64_t)t * step;
        const double2 a = F[k], b = F[k + avg], g = G[k];
        const double ax = 0.5 * (a.x + b.x), ay = 0.5 * (a.y + b.y);
        s += ax * g.x + ay * g.y;  // Re(avg * conj(g))
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) *out = scale * s;
    }
}

int launch_status(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FDFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return FDFD_OK;
}

}  // namespace
}  // namespace fdfd

using namespace fdfd;

extern "C" int fdfd_kerr_assemble(int64_t n, const void *E, const double *eps_r, const double *region,
                                  double chi, int32_t eps_scale, double eps_max, double omega, double L0,
                                  int32_t accumulate, double *eps_nl, double *dnl_deps, void *dnl_de,
                                  void *jac_diag, void *jac_off, void *stream) {
    if (n < 1 || !E || !region) return fail(FDFD_ERR_BAD_ARG, "kerr_assemble: bad size or NULL input");
    if (eps_scale && (!eps_r || !(eps_max != 1.0)))
        return fail(FDFD_ERR_BAD_ARG, "kerr_assemble: eps_scale needs eps_r and eps_max != 1");
    if (!eps_nl && !dnl_deps && !dnl_de && !jac_diag && !jac_off)
        return fail(FDFD_ERR_BAD_ARG, "kerr_assemble: no output requested");
    if (!(L0 > 0.0)) return fail(FDFD_ERR_BAD_ARG, "kerr_assemble: L0 must be positive");
    const double w2e0L = ((omega * omega) * EPSILON_0) * L0;  // simulation.py:67 / nonlinear_solvers.py:136
    const double inv_epsm1 = eps_scale ? 1.0 / (eps_max - 1.0) : 0.0;
    k_kerr_assemble<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(
        n, (const double2 *)E, eps_r, region, 3.0 * chi, eps_scale ? 1 : 0, inv_epsm1, w2e0L, accumulate ? 1 : 0,
        eps_nl, dnl_deps, (double2 *)dnl_de, (double2 *)jac_diag, (double2 *)jac_off);
    return launch_status("kerr_assemble");
}

extern "C" int fdfd_flux_probe(int32_t Nx, int32_t Ny, int32_t pol, int32_t normal, int32_t i0, int32_t j0,
                               int32_t len, double dl, const void *F, const void *G, double *out,
                               void *stream) {
    if (Nx < 2 || Ny < 2 || !F || !G || !out) return fail(FDFD_ERR_BAD_ARG, "flux_probe: bad grid or NULL buffer");
    if (pol != FDFD_POL_EZ && pol != FDFD_POL_HZ) return fail(FDFD_ERR_BAD_ARG, "flux_probe: bad pol");
    if (normal != 0 && normal != 1) return fail(FDFD_ERR_BAD_ARG, "flux_probe: normal must be 0 (x) or 1 (y)");
    if (len < 0) return fail(FDFD_ERR_BAD_ARG, "flux_probe: negative length");
    // the line and the averaging neighbour must lie inside the grid
    const bool ok = normal == 0 ? (i0 >= 0 && i0 + 1 < Nx && j0 >= 0 && j0 + len < Ny)
                                : (j0 >= 0 && j0 + 1 < Ny && i0 >= 0 && i0 + len < Nx);
    if (!ok) return fail(FDFD_ERR_BAD_ARG, "flux_probe: the probe line leaves the grid");
    const int64_t base = (int64_t)i0 * Ny + j0;
    const int64_t step = normal == 0 ? 1 : Ny, avg = normal == 0 ? Ny : 1;
    // Ez: x -> -1/2, y -> +1/2; Hz: x -> +1/2, y -> -1/2 (simulation.py:289-315)
    const double sign = (pol == FDFD_POL_EZ) == (normal == 0) ? -0.5 : 0.5;
    k_flux_line<<<1, kThreads, 0, (cudaStream_t)stream>>>((const double2 *)F, (const double2 *)G, base, step, avg,
                                                          len, dl * sign, out);
    return launch_status("flux_probe");
}
