/*
 * fdfd_gb300.h -- C ABI of the GB300 (sm_103a) FDFD engine.
 *
 * The engine replaces the hot path of fdfdpy: PML-stretched 2D Maxwell
 * operator assembly (fdfdpy/linalg.py:41-107, fdfdpy/pml.py:7-89,
 * fdfdpy/derivatives.py:7-34) followed by the complex sparse direct solve
 * (fdfdpy/linalg.py:122-149) and the field recovery that follows it
 * (fdfdpy/simulation.py:129-175).
 *
 * Conventions shared by every entry point:
 *   - Plain C types only.  Device buffers are raw pointers owned by the
 *     caller (any allocator); complex numbers are interleaved (re, im) pairs
 *     of double (complex128) unless stated otherwise.
 *   - Grids are (Nx, Ny), C order: unknown k = i*Ny + j, exactly as the
 *     reference's eps_r.reshape(-1).
 *   - Every call is ordered on the caller's CUDA stream (`stream`, a
 *     cudaStream_t passed as void*; NULL = legacy default stream).
 *   - Every call returns an int status (FDFD_OK = 0) and never throws.
 *     fdfd_last_error() gives a human-readable message for the calling
 *     thread.
 */
#ifndef FDFD_GB300_H
#define FDFD_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------- */
#define FDFD_OK                 0
#define FDFD_ERR_BAD_ARG        1   /* invalid size, pointer or option      */
#define FDFD_ERR_OOM            2   /* device allocation refused            */
#define FDFD_ERR_CUDA           3   /* a CUDA runtime call failed           */
#define FDFD_ERR_SINGULAR_PIVOT 4   /* a zero pivot was met (not replaced)  */
#define FDFD_ERR_NOT_CONVERGED  5   /* refinement hit its iteration cap     */
#define FDFD_ERR_NO_DEVICE      6   /* no CUDA device visible               */
#define FDFD_ERR_TIMEOUT        7   /* a bounded device-side wait ran out:
                                       the result of that call is not valid  */

/* ---- polarizations and precisions ------------------------------------- */
#define FDFD_POL_EZ 0
#define FDFD_POL_HZ 1

#define FDFD_PREC_C128 0   /* plain: complex128 factor                    */
#define FDFD_PREC_C64  1   /* mixed: complex64 factor + FP64 refinement   */
#define FDFD_PREC_C64_TC 2 /* mixed, Schur updates of large fronts on the
                              tcgen05 tensor cores (3xTF32 split)         */

/* Operator description.  Mirrors the arguments of construct_A
 * (fdfdpy/linalg.py:41-44).  All pointers are DEVICE pointers.
 *   eps      : (Nx*Ny) float64 relative permittivity eps_r.
 *   eps_add  : optional (Nx*Ny) float64 added to eps_r in the diagonal term
 *              only (the Kerr term of fdfdpy/simulation.py:57-68); NULL = 0.
 *   diag_add : optional (Nx*Ny) complex128 added to the operator diagonal
 *              (Newton Jacobian, fdfdpy/nonlinear_solvers.py:139-141); NULL.
 *   inv_s    : the four stretched-coordinate factors 1/s as complex128
 *              vectors: inv_sxf, inv_sxb (Nx each), inv_syf, inv_syb (Ny
 *              each), from fdfd_pml_sfactors (fdfdpy/pml.py:42-89).
 *   xlen/ylen: xrange[1]-xrange[0], yrange[1]-yrange[0] (grid spacing is
 *              xlen/Nx, ylen/Ny as in fdfdpy/linalg.py:25-33).
 *   stencil  : optional explicit 5-point operator, complex128 [5][Nx*Ny]
 *              (centre, (i-1,j), (i+1,j), (i,j-1), (i,j+1) coefficients of
 *              each row; neighbours wrap periodically).  When set, eps,
 *              omega and the PML fields are not used for the coefficients
 *              and any grid with Nx, Ny >= 1 is accepted (coupling to a
 *              neighbour that coincides with the cell itself is added to
 *              the diagonal).  The inv_s vectors may then be NULL; they are
 *              only needed for transposed solves.                        */
typedef struct fdfd_operator {
    int32_t Nx, Ny;
    int32_t pol;        /* FDFD_POL_EZ or FDFD_POL_HZ                    */
    int32_t averaging;  /* Hz only: grid-averaged eps (linalg.py:73-78)   */
    double  omega;
    double  L0;
    double  xlen, ylen;
    const double *eps;
    const double *eps_add;
    const void   *diag_add;
    const void   *inv_sxf, *inv_sxb, *inv_syf, *inv_syb;
    const void   *stencil;
} fdfd_operator;

/* ---- library ----------------------------------------------------------- */
const char *fdfd_last_error(void);
int fdfd_version(void);

/* ---- PML ---------------------------------------------------------------
 * Replaces create_sfactor + the 1/s broadcast of S_create
 * (fdfdpy/pml.py:7-39, 64-75).  Writes 1/s for one axis:
 *   out_inv_f, out_inv_b : (Nw) complex128 device vectors.
 * wlen = wrange[1]-wrange[0].                                            */
int fdfd_pml_sfactors(int32_t Nw, int32_t Nw_pml, double wlen, double omega,
                      double L0, void *out_inv_f, void *out_inv_b,
                      void *stream);

/* ---- K1: operator assembly --------------------------------------------
 * Replaces construct_A (fdfdpy/linalg.py:41-107).  Emits canonical CSR
 * (rows sorted by column): indptr (n+1, int32), indices (5n, int32),
 * data (5n complex128).  Requires Nx >= 3 and Ny >= 3.                    */
int fdfd_assemble_csr(const fdfd_operator *op, int32_t *indptr,
                      int32_t *indices, void *data, void *stream);

/* Emits one derivative operator of the reference's `derivs` dict
 * (fdfdpy/linalg.py:59-62 / 86-89, 100-105) as canonical CSR with 2 nnz
 * per row: which = 0 Dxf, 1 Dxb, 2 Dyf, 3 Dyb.                            */
int fdfd_assemble_deriv_csr(const fdfd_operator *op, int32_t which,
                            int32_t *indptr, int32_t *indices, void *data,
                            void *stream);

/* ---- K2: matrix-free FP64 residual ------------------------------------
 * r = b - A x for nrhs right-hand sides stored column after column
 * (leading dimension n).  Replaces the mat-vec used by the reference's
 * residual checks and Newton f(E) (fdfdpy/nonlinear_solvers.py:130-132). */
int fdfd_residual(const fdfd_operator *op, const void *x, const void *b,
                  void *r, int32_t nrhs, void *stream);

/* y = A x (or A^T x when transpose != 0).                                */
int fdfd_apply(const fdfd_operator *op, const void *x, void *y,
               int32_t nrhs, int32_t transpose, void *stream);

/* ---- K8: field recovery ------------------------------------------------
 * Replaces fdfdpy/simulation.py:129-175.  From the solved primary field X
 * (Ez or Hz, complex128 n) writes the two secondary fields:
 *   Ez: f1 = Hx, f2 = Hy;   Hz: f1 = Ex, f2 = Ey.                        */
int fdfd_fields(const fdfd_operator *op, const void *X, void *f1, void *f2,
                void *stream);

/* ---- mode-source slice operator ---------------------------------------
 * Writes the explicit stencil (see fdfd_operator.stencil, grid N x 1) of
 * the 1-D periodic slice operator of insert_mode minus a shift:
 *   Ez: omega^2 mu0' diag(eps0' eps) + Dxf Dxb - shift I     (mode.py:88)
 *   Hz: omega^2 mu0' T_eps + T_eps Dxf T_epsx^-1 Dxb - shift I (mode.py:91)
 * with raw periodic differences of spacing dl (mode.py:79-80) and
 * T_epsx = eps0' * grid_average(eps slice, 'x') (mode.py:83), which
 * averages along the slice only when `average` is nonzero (a slice normal
 * to y; a slice normal to x is one row, so its 'x' average is eps itself).
 * eps_slice: N float64 (device).  out: 5N complex128 (device).          */
int fdfd_mode_stencil(int32_t N, int32_t pol, int32_t average,
                      const double *eps_slice, double omega, double dl,
                      double L0, double shift, void *out, void *stream);

/* ---- K9: adjoint gradient ----------------------------------------------
 * dL/d(eps_r) for a real loss L of the solved primary field E, given the
 * adjoint field lambda = A^-T conj(dL/dE) (torch's complex gradient
 * convention), written to grad (n float64):
 *   Ez: -omega^2 * eps0 * L0 * Re(lambda * E)  (A's eps term is diagonal,
 *       fdfdpy/linalg.py:53-54,66);
 *   Hz: sum over the edge permittivities eps_x, eps_y that depend on the
 *       cell (grid-averaged, linalg.py:73-78, or not) of
 *       d eps_edge/d eps_r * Re((Df'^T lambda)(Db' E)) / eps_edge^2
 *       (A's eps terms Dxf' Tx^-1 Dxb' + Dyf' Ty^-1 Dyb', linalg.py:86-93).
 * No counterpart in the reference (it has no derivative w.r.t. eps).    */
int fdfd_adjoint_grad_eps(const fdfd_operator *op, const void *lambda_,
                          const void *E, double *grad, void *stream);

/* ---- K1-NL: Kerr terms ---------------------------------------------------
 * One pass over n cells for one Kerr nonlinearity (chi already divided by
 * L0^2, as Simulation.add_nl stores it), replacing the numpy evaluation of
 * fdfdpy/nonlinearity.py:18-34, their sum in Simulation.compute_nl
 * (fdfdpy/simulation.py:57-68) and the Jacobian terms of nl_eq_and_jac
 * (fdfdpy/nonlinear_solvers.py:117-149).  With s = (eps_r - 1)/(eps_max - 1)
 * when eps_scale != 0, else 1:
 *   eps_nl   = 3 chi region |E|^2 s                          (float64)
 *   dnl_deps = 3 chi region |E|^2 / (eps_max - 1), or 0      (float64)
 *   dnl_de   = 3 chi region conj(E) s                        (complex128)
 *   jac_diag = dAde * E,  jac_off = conj(dAde) * E           (complex128)
 *   with dAde = dnl_de * omega^2 eps0 L0.
 * Every output pointer may be NULL (not written); accumulate != 0 adds to
 * the outputs (several nonlinearities) instead of overwriting them.
 * E: complex128 (device); eps_r (needed with eps_scale), region: float64. */
int fdfd_kerr_assemble(int64_t n, const void *E, const double *eps_r,
                       const double *region, double chi, int32_t eps_scale,
                       double eps_max, double omega, double L0,
                       int32_t accumulate, double *eps_nl, double *dnl_deps,
                       void *dnl_de, void *jac_diag, void *jac_off,
                       void *stream);

/* ---- flux probe ----------------------------------------------------------
 * Replaces Simulation.flux_probe (fdfdpy/simulation.py:260-315) as a device
 * reduction over one line of cells.  normal = 0 (x): the line is
 * (i0, j0 .. j0+len-1) and F is averaged with (i0+1, j); normal = 1 (y): the
 * line is (i0 .. i0+len-1, j0), averaged with (i, j0+1).  F is the field
 * the reference averages (Ez for pol Ez, Hz for pol Hz), G its partner
 * (Hy / Hx for Ez, Ey / Ex for Hz, x / y normal).  Writes to *out (device
 * double): dl * c * sum Re(avg(F) conj(G)), c = -1/2 (Ez, x), +1/2 (Ez, y),
 * +1/2 (Hz, x), -1/2 (Hz, y).  The line and the averaging neighbour must
 * lie inside the grid (FDFD_ERR_BAD_ARG otherwise).                      */
int fdfd_flux_probe(int32_t Nx, int32_t Ny, int32_t pol, int32_t normal,
                    int32_t i0, int32_t j0, int32_t len, double dl,
                    const void *F, const void *G, double *out, void *stream);

/* ---- reductions --------------------------------------------------------
 * Column 2-norms of a complex128 (n x ncol) array, written to host array
 * out_host (ncol doubles); synchronises the stream.                      */
int fdfd_norms(const void *v, int64_t n, int32_t ncol, double *out_host,
               void *stream);

/* Same column 2-norms as fdfd_norms, computed without allocating any device
 * memory (fdfd_norms takes its partial-sum scratch from cudaMallocAsync).
 * No counterpart in the reference: it exists for callers that cannot
 * allocate at call time, such as a process whose device memory is held by
 * its own allocator under a fixed budget.
 *   - The scratch is one fixed array in the library's static device memory
 *     (about 39 KB); every GPU that loads the library holds it until exit.
 *   - At most 8 columns per call; more returns FDFD_ERR_BAD_ARG.
 *   - Every call shares the array: calls that overlap on the GPU (other
 *     streams, other threads) race and must be serialised by the caller.
 *   - Never calls cudaMalloc, cudaFree or an allocating library routine;
 *     synchronises the stream to return the result in out_host, so it
 *     cannot be called while the stream is being captured into a graph. */
int fdfd_norms_noalloc(const void *v, int64_t n, int32_t ncol,
                       double *out_host, void *stream);

/* ---- symbolic analysis (host only) ------------------------------------
 * Geometric nested dissection of the periodic Nx x Ny grid (the graph of
 * construct_A's 5-point operator) into a front tree.  Replaces the fill-
 * reducing ordering inside PARDISO/SuperLU (fdfdpy/linalg.py:134-141).  */
typedef struct fdfd_symbolic fdfd_symbolic;

typedef struct fdfd_symbolic_info {
    int32_t Nx, Ny;
    int32_t n_fronts;
    int32_t n_levels;
    int64_t sum_m;          /* total front index-list length             */
    int64_t pool_entries;   /* sum over fronts of ld*m                   */
    int64_t factor_entries; /* sum p^2 + 2 p (m-p): stored L+U entries   */
    double  factor_flops;   /* real flops of the complex partial LUs     */
    int32_t max_m, max_p;
} fdfd_symbolic_info;

int fdfd_symbolic_create(int32_t Nx, int32_t Ny, int32_t leaf_area,
                         fdfd_symbolic **out);
/* A batch symbolic: `batch` copies of the Nx x Ny front tree as one forest,
 * for factoring `batch` operators of the same grid in one pass (every
 * level's launches cover the fronts of all of them).  Problem b's unknowns
 * are [b n, (b + 1) n), n = Nx Ny; vectors are the problems' vectors one
 * after the other, and the info's Nx is batch * Nx.  No counterpart in
 * fdfdpy (it serves many independent solver_direct calls at once). */
int fdfd_symbolic_create_batch(int32_t Nx, int32_t Ny, int32_t leaf_area,
                               int32_t batch, fdfd_symbolic **out);
int fdfd_symbolic_info_get(const fdfd_symbolic *sym, fdfd_symbolic_info *info);
/* Copies one host array out (tests and diagnostics).  which:
 *  0 front p (n_fronts int32)     1 front m          2 front parent
 *  3 front child0                 4 front child1     5 front height
 *  6 front vars_off (int32)       7 level_ptr (n_levels+1 int32)
 *  8 vars (sum_m int32)           9 relmap (sum_m int32)
 * 10 nbr_loc (4n int32)          11 var_front (n)   12 var_loc (n)
 * 13 front ld (int32)            14 pool_off (n_fronts int64)           */
int fdfd_symbolic_export(const fdfd_symbolic *sym, int32_t which, void *dst);
void fdfd_symbolic_destroy(fdfd_symbolic *sym);

/* ---- numeric factorization ---------------------------------------------
 * Multifrontal LU of the operator over the symbolic front tree, without
 * pivoting (static pivots; tiny pivots are replaced and counted).
 * Replaces pardisoSolver(A, mtype=13).factor() (fdfdpy/linalg.py:135-136)
 * and the factor inside spsolve (linalg.py:141).  The factor owns its
 * device memory (allocated on the current device at create time).        */
typedef struct fdfd_factor fdfd_factor;

typedef struct fdfd_factor_stats {
    int32_t tiny_pivots;    /* pivots replaced by the static threshold   */
    int32_t refine_iters;   /* refinement steps of the last solve        */
    double  rel_residual;   /* ||b - A x|| / ||b|| of the last solve (max */
                            /* over right-hand sides)                     */
    double  factor_ms;      /* device time of the last factorization     */
    double  solve_ms;       /* device time of the last solve             */
    int32_t tc_errors;      /* tensor-core tiles that timed out (0)       */
    int32_t pad;
} fdfd_factor_stats;

int fdfd_factor_bytes(const fdfd_symbolic *sym, int32_t precision,
                      int32_t max_nrhs, int64_t *bytes);
int fdfd_factor_create(fdfd_symbolic *sym, int32_t precision,
                       int32_t max_nrhs, fdfd_factor **out);
/* Returns FDFD_ERR_TIMEOUT (after synchronising the stream) when a bounded
 * wait of the tensor-core Schur update ran out; the factor then holds no
 * valid values until the next successful call.                          */
int fdfd_factor_numeric(fdfd_factor *fac, const fdfd_operator *op,
                        void *stream);
/* One application of the factor: x = A^-1 b (transpose = 0) or
 * x = A^-T b (transpose = 1), complex128 in and out, nrhs columns.
 * Synchronises the stream to read the substitutions' wait status and
 * returns FDFD_ERR_TIMEOUT when one of their bounded waits ran out.      */
int fdfd_factor_solve(fdfd_factor *fac, const void *b, void *x,
                      int32_t nrhs, int32_t transpose, void *stream);
/* Solve with FP64 iterative refinement against the operator `op` until
 * max_j ||b_j - A x_j|| / ||b_j|| <= tol or max_iter steps.  When `op`
 * describes the factored operator (same grid, scalars and device buffers
 * as at fdfd_factor_numeric) the residual reads the operator coefficients
 * stored by fdfd_factor_numeric (operator buffers changed in place since
 * then need a new fdfd_factor_numeric); any other operator is applied
 * matrix-free.  Replaces solver_direct (fdfdpy/linalg.py:122-149).
 * Returns FDFD_ERR_NOT_CONVERGED (x still written) when tol was not
 * reached, FDFD_ERR_TIMEOUT when a bounded wait of the substitutions ran
 * out (x not valid).                                                     */
int fdfd_solve_refined(fdfd_factor *fac, const fdfd_operator *op,
                       const void *b, void *x, int32_t nrhs,
                       int32_t transpose, double tol, int32_t max_iter,
                       void *stream);
/* Static-pivot threshold, relative to max|diag(A)| (the factor works on A
 * scaled by 1/max|diag(A)|): a pivot of smaller modulus is lifted to it and
 * counted in tiny_pivots.  -1 restores the default (1e-5 for complex64,
 * sqrt(eps) = 1.5e-8 for complex128).  Takes effect at the next
 * fdfd_factor_numeric.                                                   */
int fdfd_factor_set_pivot_tol(fdfd_factor *fac, double rel_tol);
/* Largest front size m that is factored by one launch per level (all of
 * a level's fronts must have at most 64 pivots; the dense front is held in
 * shared memory, which also bounds m).  -1 (default): as large as
 * shared memory allows on levels of fewer than 2048 fronts, 128 on wider
 * levels; 0: never (every front goes through the per-panel kernels).
 * Takes effect at the next fdfd_factor_numeric.  No counterpart in
 * fdfdpy.                                                                */
int fdfd_factor_set_fused_limit(fdfd_factor *fac, int32_t max_m);
/* Batch factors (a factor created on a batch symbolic): factor `count` =
 * batch operators of the symbolic's grid (ops[b] for problem b) in one
 * forest factorization.  The batch shares one scaling and one static-pivot
 * threshold (relative to the largest diagonal entry of the batch), so it is
 * meant for operators of the same grid, polarization and frequency that
 * differ in eps_r.  The coefficients are evaluated at this call; the
 * operators' buffers are not read afterwards.                           */
int fdfd_factor_numeric_batch(fdfd_factor *fac, const fdfd_operator *ops,
                              int32_t count, void *stream);
/* FP64 iterative refinement of the batch: b and x hold nrhs columns of
 * batch * n entries (column r, problem p at offset (r batch + p) n); every
 * (column, problem) segment is refined until its ||b - A x|| <= tol ||b||
 * against the factored operators (FDFD_ERR_NOT_CONVERGED otherwise, x
 * still written).  rel_residuals (host, nrhs * batch doubles, optional)
 * receives the final relative residual of segment r batch + p; a zero
 * segment (a problem with fewer right-hand sides) stays zero.           */
int fdfd_solve_refined_batch(fdfd_factor *fac, const void *b, void *x,
                             int32_t nrhs, double tol, int32_t max_iter,
                             double *rel_residuals, void *stream);
/* on != 0 (default): the factorization's launch sequence is captured as a
 * CUDA graph at the first fdfd_factor_numeric(_batch) of this factor and
 * replayed by the later ones (only the evaluation of the operator's
 * coefficients runs outside it), which takes the host's launch overhead
 * off small grids.  Not used while kernel-class profiling is enabled or for
 * an explicit-stencil operator.  on = 0: direct launches.  No counterpart
 * in fdfdpy.                                                             */
int fdfd_factor_set_graphs(fdfd_factor *fac, int32_t on);
/* Polls a bounded wait of the cooperative substitutions (grid barrier,
 * published panel values) makes before it gives up and the call returns
 * FDFD_ERR_TIMEOUT; -1 restores the built-in limits (2^24 barrier polls,
 * 2^22 value polls, each with a short sleep).  For callers that want a
 * shorter failure detection, and for tests of that path.  Takes effect at
 * the next solve.  No counterpart in fdfdpy.                             */
int fdfd_factor_set_wait_limit(fdfd_factor *fac, int64_t polls);
/* One right-hand side by restarted GMRES(restart) in FP64, right-
 * preconditioned by the factor; stops at ||b - A x|| <= tol ||b|| or after
 * max_iter factor applications (FDFD_ERR_NOT_CONVERGED, x still written).
 * Same result contract as fdfd_solve_refined, usually with fewer factor
 * applications for a complex64 factor.  Allocates its Krylov workspace
 * (2 * restart + 2 vectors) on first use.                                 */
int fdfd_solve_gmres(fdfd_factor *fac, const fdfd_operator *op, const void *b,
                     void *x, int32_t transpose, double tol, int32_t max_iter,
                     int32_t restart, void *stream);
int fdfd_factor_stats_get(const fdfd_factor *fac, fdfd_factor_stats *st);
/* Copies the factor's stored operator coefficients, complex128 [5][n]
 * (the centre, then the (i-1, j), (i+1, j), (i, j-1), (i, j+1) neighbours
 * of cell k = i Ny + j; n = Nx Ny), into dst (device memory, 80 n bytes),
 * ordered on `stream`.  Valid after fdfd_factor_numeric of an operator
 * given by eps and the 1/s vectors (not an explicit stencil), else
 * FDFD_ERR_BAD_ARG.  For tests and diagnostics: the entries are those of
 * row k of construct_A (fdfd_assemble_csr).  No counterpart in fdfdpy. */
int fdfd_factor_coef_get(const fdfd_factor *fac, void *dst, void *stream);
void fdfd_factor_destroy(fdfd_factor *fac);

/* ---- profiling -----------------------------------------------------------
 * Launch counters per kernel class are always kept; CUDA-event timing of
 * each class is recorded while enabled.  Classes: 0 front assembly,
 * 1 extend-add, 2 diagonal-block LU, 3 panel TRSM, 4 Schur GEMM on the
 * tensor cores, 5 forward solve, 6 backward solve, 7 residual / norms /
 * scaling, 8 Schur GEMM in SIMT form (fronts below 192 rows, complex128,
 * complex64 without tensor cores).
 * Replaces the `timing=` prints of the reference (fdfdpy/linalg.py:131-147).
 * Not thread-safe: profile one stream at a time.                         */
int fdfd_profile_enable(int32_t on);
int fdfd_profile_reset(void);
/* Synchronises on the recorded events; writes nclass (<= 9) entries.     */
int fdfd_profile_read(int32_t nclass, double *ms, int64_t *launches);

#ifdef __cplusplus
}
#endif
#endif /* FDFD_GB300_H */
