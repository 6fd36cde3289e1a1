"""Adjoint gradient (backward = transposed solve on the forward factor +
the K9 gradient kernel) against central finite differences and a float64
CPU reference gradient (oracle: SuperLU solves with A and A^T).

The adjoint workload: Ez, 600 x 600, NPML [20, 20], centred 200 x 200
design region with eps_r ~ U[1, 12] (seed 0), background 1, point source
at (100, 300), J = |Ez(500, 300)|^2; FD step 1e-4 on 64 random design
pixels.  Bar: ||grad_adj - grad_fd|| / ||grad_fd|| <= 1e-6 over the
sampled pixels (norm-wise).
"""
import numpy as np
import pytest
import torch

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def _design(N=600, region=200, seed=0):
    rng = np.random.default_rng(seed)
    eps = np.ones((N, N))
    a = (N - region) // 2
    eps[a:a + region, a:a + region] = rng.uniform(1, 12, size=(region, region))
    mask = np.zeros((N, N), bool)
    mask[a:a + region, a:a + region] = True
    return eps, mask, rng


def test_gradient_small_matches_oracle_and_fd():
    from fdfdpy_gb300.adjoint import solve_ez
    Nx, Ny, dl = 40, 36, 0.02
    rng = np.random.default_rng(3)
    eps = 1 + 11 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[8, 18] = 1
    k = (30, 18)
    e = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
    s = torch.tensor(src, dtype=torch.float64, device="cuda", requires_grad=True)
    E = solve_ez(e, s, OMEGA, dl, [6, 6])
    J = E[k].abs() ** 2
    J.backward()
    g = e.grad.cpu().numpy().reshape(-1)
    # float64 CPU reference gradient
    A = O.construct_A(OMEGA, Nx * dl, Ny * dl, eps, [6, 6], "Ez", 1e-6)
    Eo = O.solve(A, 1j * OMEGA * src.reshape(-1))
    go = np.zeros(Nx * Ny, complex)
    go[k[0] * Ny + k[1]] = 2 * Eo[k[0] * Ny + k[1]]
    gref = O.adjoint_grad_eps_Ez(A, Eo, go, OMEGA, 1e-6)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) < 1e-9
    # source gradient: dJ/dsrc = Re(1j omega lambda)
    lam = np.linalg.solve(A.T.toarray(), np.conj(go))
    assert np.linalg.norm(s.grad.cpu().numpy().reshape(-1) - np.real(1j * OMEGA * lam)) <= 1e-9 * np.linalg.norm(
        np.real(1j * OMEGA * lam))


def test_adjoint_workload_600_against_finite_differences():
    from fdfdpy_gb300.adjoint import solve_ez
    eps, mask, rng = _design()
    N = eps.shape[0]
    src = np.zeros((N, N))
    src[100, 300] = 1
    e = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
    s = torch.tensor(src, dtype=torch.float64, device="cuda")
    E = solve_ez(e, s, OMEGA, 0.02, [20, 20], tol=1e-13)
    J = E[500, 300].abs() ** 2
    J.backward()
    grad = e.grad.cpu().numpy()
    pix = np.flatnonzero(mask.reshape(-1))
    pix = rng.choice(pix, 64, replace=False)
    h = 1e-4
    fd = []
    with torch.no_grad():
        for p in pix:
            vals = []
            for d in (h, -h):
                ep = eps.copy()
                ep.reshape(-1)[p] += d
                Ep = solve_ez(torch.tensor(ep, device="cuda"), s, OMEGA, 0.02, [20, 20], tol=1e-13)
                vals.append(float(Ep[500, 300].abs() ** 2))
            fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    adj = grad.reshape(-1)[pix]
    err = np.linalg.norm(adj - fd) / np.linalg.norm(fd)
    assert err < 1e-6, err
    # gradient outside the design region is the same formula; inside it is
    # what the optimisation uses -- both finite
    assert np.isfinite(grad).all()


def test_mixed_precision_gradient_agrees_with_plain():
    from fdfdpy_gb300.adjoint import solve_ez
    eps, mask, rng = _design(N=200, region=80, seed=1)
    src = np.zeros_like(eps)
    src[40, 100] = 1
    grads = []
    for prec in ("c128", "c64"):
        e = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
        E = solve_ez(e, torch.tensor(src, device="cuda"), OMEGA, 0.02, [20, 20], precision=prec, tol=1e-12)
        (E[160, 100].abs() ** 2).backward()
        grads.append(e.grad.cpu().numpy())
    assert np.linalg.norm(grads[1] - grads[0]) / np.linalg.norm(grads[0]) < 1e-8
