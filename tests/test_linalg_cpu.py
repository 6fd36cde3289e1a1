"""Host logic of the drop-in linalg module: recognising the periodic
5-point pattern of construct_A in an arbitrary scipy matrix (solver_direct
on a general A, fdfdpy/linalg.py:122-149) and reading its five diagonals."""
import numpy as np
import scipy.sparse as sp

from oracle import fdfd_oracle as O
from fdfdpy_gb300.linalg import stencil_of_csr

OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def test_stencil_of_csr_reads_the_five_diagonals():
    rng = np.random.default_rng(0)
    for Nx, Ny, pol in ((7, 5, "Hz"), (3, 3, "Ez"), (12, 31, "Ez")):
        eps = 1 + rng.random((Nx, Ny))
        A = O.construct_A(OMEGA, Nx * 0.02, Ny * 0.02, eps, [1, 1], pol, 1e-6)
        d = rng.random(Nx * Ny)
        got = stencil_of_csr((A + sp.diags(d)).tocoo())        # any sparse format, unsorted rows
        assert got is not None and got[:2] == (Nx, Ny)
        want = O.stencil(OMEGA, Nx * 0.02, Ny * 0.02, eps, [1, 1], pol, 1e-6)
        assert np.array_equal(got[2][0], want[0].reshape(-1) + d)
        for k in range(1, 5):
            assert np.array_equal(got[2][k], want[k].reshape(-1))


def test_stencil_of_csr_rejects_other_patterns():
    rng = np.random.default_rng(1)
    eps = 1 + rng.random((9, 8))
    A = O.construct_A(OMEGA, 0.18, 0.16, eps, [1, 1], "Ez", 1e-6).tolil()
    A[20, 50] = 1.0                                   # one entry outside the pattern
    assert stencil_of_csr(A.tocsr()) is None
    assert stencil_of_csr(sp.eye(72, format="csr")) is None
    assert stencil_of_csr(np.eye(72)) is None          # dense input: not a sparse operator
    assert stencil_of_csr(sp.random(72, 60, 0.1, format="csr")) is None
