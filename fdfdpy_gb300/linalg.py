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


def solver_direct(A, b, timing=False, solver=DEFAULT_SOLVER, precision=DEFAULT_PRECISION, tol=None,
                  max_iter=None):
    """x = A^-1 b (fdfdpy/linalg.py:122-149) by the GPU multifrontal LU.

    ``A`` must come from ``construct_A`` (it carries its device operator).
    An all-zero b returns float zeros, as the reference does."""
    if solver.lower() not in ('pardiso', 'scipy'):
        raise ValueError('Invalid solver choice: {}, options are pardiso or scipy'.format(str(solver)))
    b = np.asarray(b).astype(np.complex128).reshape((-1,))
    if not b.any():
        return np.zeros(b.shape)
    op = getattr(A, 'fdfd_operator', None)
    if op is None:
        raise TypeError("solver_direct: A must be built by fdfdpy_gb300 construct_A (its device "
                        "operator is attached as A.fdfd_operator)")
    t = time()
    fac = engine.Factor(engine.symbolic_for(op.Nx, op.Ny), precision).numeric(op)
    x = fac.solve(b, tol=DEFAULT_TOL[precision] if tol is None else tol,
                  max_iter=DEFAULT_MAX_REFINE[precision] if max_iter is None else max_iter)
    x = x.cpu().numpy()
    if timing:
        print('Linear system solve took {:.2f} seconds'.format(time() - t))
    return x
