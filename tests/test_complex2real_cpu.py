"""The real-linear Newton system J11 d + J12 conj(d) = f (the reference's
solver_complex2real, fdfdpy/linalg.py:152-186) solved by the host GMRES of
nonlinear_solvers.solve_complex2real with an approximate complex inverse
of J11 as preconditioner -- checked on CPU tensors against the real 2n x 2n
solve, including a J12 strong enough that a fixed-point refinement with the
same preconditioner diverges."""
import numpy as np
import torch

from fdfdpy_gb300.nonlinear_solvers import solve_complex2real


class _Op:
    def __init__(self, M):
        self.M = M

    def apply(self, x, transpose=False):
        return (self.M.T if transpose else self.M) @ x


class _ApproxInverse:
    """x -> inv(J11 + E) x: a perturbed inverse, like a complex64 factor."""

    def __init__(self, M, rng, eps):
        M = M.numpy()
        n = M.shape[0]
        E = eps * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * np.abs(M).max()
        self.Minv = torch.from_numpy(np.linalg.inv(M + E))

    def apply_inverse(self, v, transpose=False):
        return (self.Minv.T if transpose else self.Minv) @ v


def _real2n(J11, J12, f):
    A = np.block([[J11.real + np.diag(J12.real), -J11.imag + np.diag(J12.imag)],
                  [J11.imag + np.diag(J12.imag), J11.real - np.diag(J12.real)]])
    z = np.linalg.solve(A, np.concatenate([f.real, f.imag]))
    n = f.size
    return z[:n] + 1j * z[n:]


def test_complex2real_gmres_matches_real_solve():
    rng = np.random.default_rng(7)
    n = 120
    J11 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 12 * np.eye(n)
    for strength in (0.1, 4.0):
        J12 = strength * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
        f = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        ref = _real2n(J11, J12, f)
        M = torch.from_numpy(J11)
        fac = _ApproxInverse(M, rng, 1e-4)
        d, rel, it = solve_complex2real(fac, _Op(M), torch.from_numpy(J12), torch.from_numpy(f), tol=1e-12,
                                        max_iter=400, restart=40)
        d = d.numpy()
        assert rel <= 1e-12, (strength, rel, it)
        assert np.linalg.norm(d - ref) <= 1e-9 * np.linalg.norm(ref), strength
        # the fixed-point iteration with the same preconditioner diverges for strong J12
        if strength >= 4.0:
            x = fac.apply_inverse(torch.from_numpy(f))
            Jd = lambda v: M @ v + torch.from_numpy(J12) * torch.conj(v)
            r0 = float(torch.linalg.vector_norm(torch.from_numpy(f) - Jd(x)))
            for _ in range(20):
                x = x + fac.apply_inverse(torch.from_numpy(f) - Jd(x))
            assert float(torch.linalg.vector_norm(torch.from_numpy(f) - Jd(x))) > r0


def test_complex2real_zero_rhs():
    n = 8
    M = torch.eye(n, dtype=torch.complex128)
    d, rel, it = solve_complex2real(type("F", (), {"apply_inverse": lambda self, v, transpose=False: v})(), _Op(M),
                                    torch.zeros(n, dtype=torch.complex128), torch.zeros(n, dtype=torch.complex128))
    assert it == 0 and rel == 0.0 and not d.any()


def test_complex2real_transposed_system():
    """transpose=True solves J11^T d + J12 conj(d) = f (the Kerr adjoint)
    with the transposed preconditioner."""
    rng = np.random.default_rng(8)
    n = 90
    J11 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 12 * np.eye(n)
    J12 = 3.0 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    f = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = _real2n(J11.T, J12, f)
    M = torch.from_numpy(J11)
    d, rel, it = solve_complex2real(_ApproxInverse(M, rng, 1e-4), _Op(M), torch.from_numpy(J12), torch.from_numpy(f),
                                    tol=1e-12, max_iter=400, restart=40, transpose=True)
    assert rel <= 1e-12 and np.linalg.norm(d.numpy() - ref) <= 1e-9 * np.linalg.norm(ref)
