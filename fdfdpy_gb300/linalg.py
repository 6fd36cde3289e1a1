"""Drop-in counterparts of fdfdpy/linalg.py, backed by the GPU engine.

``construct_A`` assembles on the GPU (K1) and returns host scipy CSR
matrices as the reference does; the matrix carries the device operator
(``A.fdfd_operator``) so that ``solver_direct`` can factor it on the GPU.
"""
from __future__ import annotations

from time import time

import numpy as np

from . import engine
from .constants import (DEFAULT_MATRIX_FORMAT, DEFAULT_SOLVER, DEFAULT_PRECISION, DEFAULT_TOL,
                        DEFAULT_MAX_REFINE)


def grid_average(center_array, w):
    """Values at cell edges: (roll(a, 1, axis) + a) / 2 (fdfdpy/linalg.py:16-22)."""
    xy = {'x': 0, 'y': 1}
    return (np.roll(center_array, 1, axis=xy[w]) + center_array) / 2


def dL(N, xrange, yrange=None):
    """Grid spacing (xrange[1]-xrange[0]) / N (fdfdpy/linalg.py:25-33)."""
    if yrange is None:
        L = np.array([np.diff(xrange)[0]])
    else:
        L = np.array([np.diff(xrange)[0], np.diff(yrange)[0]])
    return L / N


def is_equal(matrix1, matrix2):
    """Sparse equality (fdfdpy/linalg.py:36-38)."""
    return (matrix1 != matrix2).nnz == 0


def construct_A(omega, xrange, yrange, eps_r, NPML, pol, L0, averaging=True, timing=False,
                matrix_format=DEFAULT_MATRIX_FORMAT):
    """(A, derivs) of fdfdpy/linalg.py:41-107, assembled on the GPU.

    A is returned in canonical CSR (columns sorted within each row; the
    reference's rows are unsorted but hold the same entries)."""
    if pol not in ('Ez', 'Hz'):
        raise ValueError("something went wrong and pol is not one of Ez, Hz, instead was given {}".format(pol))
    t = time()
    op = engine.DeviceOperator(omega, eps_r, xrange[1] - xrange[0], yrange[1] - yrange[0], NPML, pol,
                               L0, averaging=averaging)
    A = op.csr()
    derivs = {name: op.deriv_csr(name) for name in ('Dyb', 'Dxb', 'Dxf', 'Dyf')}
    if matrix_format != 'csr':
        A = A.asformat(matrix_format)
        derivs = {k: v.asformat(matrix_format) for k, v in derivs.items()}
    A.fdfd_operator = op
    if timing:
        print('construct_A took {:.4f} seconds'.format(time() - t))
    return (A, derivs)


def stencil_of_csr(A):
    """(Nx, Ny, [5][n] coefficients) of a sparse matrix with the periodic
    5-point pattern of construct_A (every row k = i Ny + j couples to
    (i -+ 1, j) and (i, j -+ 1) modulo the grid, linalg.py:41-107 and
    derivatives.py:22-32) -- e.g. A + Anl of simulation.py:125 or any
    operator a user assembled on that grid -- or None for another pattern.
    The grid is read off row 0, whose columns are {0, 1, Ny-1, Ny, n-Ny}."""
    import scipy.sparse as sp
    if not sp.issparse(A) or A.shape[0] != A.shape[1]:
        return None
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.sort_indices()
    n = A.shape[0]
    row0 = A.indices[A.indptr[0]:A.indptr[1]]
    if n < 9 or len(row0) != 5:
        return None
    Ny = int(row0[3])
    if Ny < 3 or n % Ny or n // Ny < 3 or list(row0) != [0, 1, Ny - 1, Ny, n - Ny]:
        return None
    Nx = n // Ny
    i, j = np.divmod(np.arange(n), Ny)
    cols = np.stack([i * Ny + j, ((i - 1) % Nx) * Ny + j, ((i + 1) % Nx) * Ny + j,
                     i * Ny + (j - 1) % Ny, i * Ny + (j + 1) % Ny])
    vals = np.asarray(A[np.tile(np.arange(n), 5), cols.reshape(-1)]).reshape(5, n).astype(np.complex128)
    if np.count_nonzero(vals) != A.count_nonzero():
        return None                                 # entries outside the 5-point pattern
    return Nx, Ny, vals


def solver_direct(A, b, timing=False, solver=DEFAULT_SOLVER, precision=DEFAULT_PRECISION, tol=None,
                  max_iter=None):
    """x = A^-1 b (fdfdpy/linalg.py:122-149) by the GPU multifrontal LU.

    ``A`` from ``construct_A`` carries its device operator and is factored
    from it; any other sparse matrix with the periodic 5-point pattern of
    that operator (for instance ``A + Anl``, simulation.py:125) is factored
    from its five diagonals; other matrices raise ValueError.  An all-zero
    b returns float zeros, as the reference does."""
    if solver.lower() not in ('pardiso', 'scipy'):
        raise ValueError('Invalid solver choice: {}, options are pardiso or scipy'.format(str(solver)))
    b = np.asarray(b).astype(np.complex128).reshape((-1,))
    if not b.any():
        return np.zeros(b.shape)
    t = time()
    op = getattr(A, 'fdfd_operator', None)
    if op is None:
        st = stencil_of_csr(A)
        if st is None:
            raise ValueError("solver_direct: the GPU engine factors the periodic 5-point operator of "
                             "construct_A; this matrix has another sparsity pattern")
        if A.shape[0] != b.size:
            raise ValueError("solver_direct: A and b have different sizes")
        Nx, Ny, vals = st
        op = engine.StencilOperator(Nx, Ny, engine.as_c128(vals))
    fac = engine.Factor(engine.symbolic_for(op.Nx, op.Ny), precision).numeric(op)
    x = fac.solve(b, tol=DEFAULT_TOL[precision] if tol is None else tol,
                  max_iter=DEFAULT_MAX_REFINE[precision] if max_iter is None else max_iter)
    x = x.cpu().numpy()
    if timing:
        print('Linear system solve took {:.2f} seconds'.format(time() - t))
    return x
