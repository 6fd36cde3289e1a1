"""GPU parity of the stencil kernels against the golden vectors and the
oracle: PML stretch factors, CSR assembly (K1), derivative operators, the
matrix-free residual (K2) and field recovery (K8).

Bars: indices/indptr bit-exact; values within 1e-14 relative per entry
(bit-exact is reported and expected for these kernels); fields within
1e-13 relative in norm.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


@pytest.fixture(scope="module")
def eng():
    from fdfdpy_gb300 import engine
    engine.device()
    return engine


def _small_cases():
    g = np.load(GOLD / "small_ops.npz")
    names = sorted({k[:-5] for k in g.files if k.endswith("_args")})
    return g, names


def test_sfactors_bitexact(eng):
    from fdfdpy_gb300 import _native as N
    sf = np.load(GOLD / "sfactors.npz")
    for t in "abcde":
        wlen, Nw, npml, om, L0 = sf[t + "_args"]
        Nw, npml = int(Nw), int(npml)
        f = torch.empty(Nw, dtype=torch.complex128, device="cuda")
        b = torch.empty(Nw, dtype=torch.complex128, device="cuda")
        N.call("fdfd_pml_sfactors", Nw, npml, float(wlen), float(om), float(L0), C.c_void_p(f.data_ptr()),
               C.c_void_p(b.data_ptr()), eng.stream_ptr())
        for got, s in ((f, "f"), (b, "b")):
            want = 1 / sf[f"{t}_{s}"]
            got = got.cpu().numpy()
            rel = np.max(np.abs(got - want) / np.abs(want))
            # x**4 differs from glibc's pow by at most an ulp on rare inputs
            assert rel <= 5e-16, (t, s, rel)


@pytest.mark.parametrize("averaging", [True, False])
def test_csr_matches_reference(eng, averaging):
    g, names = _small_cases()
    for nm in names:
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny = int(Nx), int(Ny)
        pol = "Ez" if pol == 0 else "Hz"
        if not averaging and pol == "Ez":
            continue
        op = eng.DeviceOperator(om, g[nm + "_eps"], Nx * dl, Ny * dl, [int(p0), int(p1)], pol, L0,
                                averaging=averaging)
        A = op.csr()
        assert np.array_equal(A.indptr, g[nm + "_indptr"])
        assert np.array_equal(A.indices, g[nm + "_indices"])
        want = g[nm + "_data"] if averaging else g[nm + "_noavg_data"]
        rel = np.max(np.abs(A.data - want) / np.abs(want))
        assert rel <= 1e-14, (nm, rel)
        for dn in ("Dxf", "Dxb", "Dyf", "Dyb"):
            D = op.deriv_csr(dn)
            want = g[f"{nm}_{dn}"]
            assert np.max(np.abs(D.data - want) / np.abs(want)) <= 1e-15, (nm, dn)


def test_csr_200_ez_matches_reference_rows(eng):
    g = np.load(GOLD / "ez200.npz")
    N = 200
    eps = np.ones((N, N))
    eps[80:120, 80:120] = 12
    op = eng.DeviceOperator(OMEGA, eps, N * 0.02, N * 0.02, [15, 15], "Ez", 1e-6)
    A = op.csr()
    rows = g["rows"]
    got_idx = np.stack([A.indices[A.indptr[r]:A.indptr[r + 1]] for r in rows])
    got = np.stack([A.data[A.indptr[r]:A.indptr[r + 1]] for r in rows])
    assert np.array_equal(got_idx, g["row_indices"])
    assert np.max(np.abs(got - g["row_data"]) / np.abs(g["row_data"])) <= 1e-14
    assert abs(np.abs(A.data).sum() - g["data_abs_sum"]) / g["data_abs_sum"] < 1e-14


@pytest.mark.parametrize("N,pol", [(2048, "Hz"), (1024, "Ez")])
def test_csr_full_size_matches_oracle(eng, N, pol):
    rng = np.random.default_rng(0)
    eps = np.kron(rng.choice([1.0, 12.25], size=(N // 16, N // 16)), np.ones((16, 16)))
    dl = 0.01
    op = eng.DeviceOperator(OMEGA, eps, N * dl, N * dl, [20, 20], pol, 1e-6)
    indptr, indices, data = op.csr_device()
    A = O.construct_A(OMEGA, N * dl, N * dl, eps, [20, 20], pol, 1e-6)
    assert torch.equal(indices.cpu(), torch.from_numpy(A.indices))
    d = data.cpu().numpy()
    assert np.max(np.abs(d - A.data) / np.abs(A.data)) <= 1e-14
    assert int(indptr[-1]) == 5 * N * N


def test_residual_and_apply(eng):
    g, names = _small_cases()
    rng = np.random.default_rng(3)
    for nm in names:
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny = int(Nx), int(Ny)
        pol = "Ez" if pol == 0 else "Hz"
        eps = g[nm + "_eps"]
        op = eng.DeviceOperator(om, eps, Nx * dl, Ny * dl, [int(p0), int(p1)], pol, L0)
        A = O.construct_A(om, Nx * dl, Ny * dl, eps, [int(p0), int(p1)], pol, L0)
        n = Nx * Ny
        x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
        b = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
        r = op.residual(x, b).cpu().numpy()
        for k in range(2):
            want = b[k] - A @ x[k]
            assert np.linalg.norm(r[k] - want) / np.linalg.norm(want) < 1e-13
            y = op.apply(x[k]).cpu().numpy()
            assert np.linalg.norm(y - A @ x[k]) / np.linalg.norm(A @ x[k]) < 1e-13
            yt = op.apply(x[k], transpose=True).cpu().numpy()
            assert np.linalg.norm(yt - A.T @ x[k]) / np.linalg.norm(A.T @ x[k]) < 1e-13


def test_fields_kernel_matches_reference(eng):
    g, names = _small_cases()
    for nm in names:
        if nm == "ez_12x9_L0":
            continue  # near-singular static case: the solved fields are not a pin
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny = int(Nx), int(Ny)
        pol = "Ez" if pol == 0 else "Hz"
        op = eng.DeviceOperator(om, g[nm + "_eps"], Nx * dl, Ny * dl, [int(p0), int(p1)], pol, L0)
        X = g[nm + "_f3"].reshape(-1)
        f1, f2 = op.fields(X)
        for got, key in ((f1, "_f1"), (f2, "_f2")):
            want = g[nm + key].reshape(-1)
            got = got.cpu().numpy()
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-14, (nm, key)
        if pol == "Hz":
            f1, f2 = op.fields(X, averaging=False)
            for got, key in ((f1, "_noavg_f1"), (f2, "_noavg_f2")):
                want = g[nm + key].reshape(-1)
                assert np.linalg.norm(got.cpu().numpy() - want) / np.linalg.norm(want) < 1e-14


def test_norms(eng):
    rng = np.random.default_rng(5)
    v = rng.standard_normal((3, 100003)) + 1j * rng.standard_normal((3, 100003))
    got = eng.norms(torch.from_numpy(v).cuda(), 100003)
    assert np.allclose(got, np.linalg.norm(v, axis=1), rtol=1e-13)


def test_bad_arguments_raise(eng):
    from fdfdpy_gb300 import _native as N
    with pytest.raises(ValueError):
        eng.DeviceOperator(OMEGA, np.ones((2, 5)), 1, 1, [0, 0], "Ez", 1e-6)
    with pytest.raises(ValueError):
        eng.DeviceOperator(OMEGA, np.ones((5, 5)), 1, 1, [0, 0], "Ex", 1e-6)
    op = N.Operator()
    op.Nx, op.Ny, op.pol = 4, 4, 0
    assert N.lib().fdfd_assemble_csr(C.byref(op), None, None, None, None) == N.FDFD_ERR_BAD_ARG


@pytest.mark.parametrize("shape,pol,averaging,kerr", [
    ((48, 40, 0.02, (8, 6)), "Ez", True, False),
    ((48, 40, 0.02, (8, 6)), "Hz", True, True),
    ((37, 300, 0.01, (5, 20)), "Hz", True, False),
    ((37, 300, 0.01, (5, 20)), "Hz", False, True),
    ((100, 513, 0.01, (10, 10)), "Ez", True, True),
    ((257, 256, 0.01, (20, 20)), "Hz", True, False),
])
def test_factor_coefficients_equal_construct_A(eng, shape, pol, averaging, kerr):
    """The coefficient store a factorization evaluates (k_coef: tiled, the
    sign-symmetric forms, 1/eps shared between neighbouring cells) holds
    exactly the entries of construct_A's rows (K1, cell by cell), in every
    direction, with ragged column blocks, both polarizations, with and
    without averaging and a Kerr term."""
    Nx, Ny, dl, npml = shape
    rng = np.random.default_rng(Nx * Ny)
    eps = np.kron(rng.choice([1.0, 12.25], size=(-(-Nx // 4), -(-Ny // 4))), np.ones((4, 4)))[:Nx, :Ny]
    eps_add = torch.from_numpy(rng.random((Nx, Ny))).cuda() if kerr else None
    op = eng.DeviceOperator(OMEGA, eps, Nx * dl, Ny * dl, list(npml), pol, 1e-6, averaging=averaging,
                            eps_add=eps_add)
    indptr, indices, data = op.csr_device()
    fac = eng.Factor(eng.symbolic_for(Nx, Ny), "c64").numeric(op)
    coef = fac.coefficients()
    n = Nx * Ny
    k = torch.arange(n, device=coef.device)
    i, j = k // Ny, k % Ny
    cols = torch.stack([k, ((i - 1) % Nx) * Ny + j, ((i + 1) % Nx) * Ny + j, i * Ny + (j - 1) % Ny,
                        i * Ny + (j + 1) % Ny])
    assert torch.equal(indptr[1:] - indptr[:-1], torch.full((n,), 5, dtype=indptr.dtype, device=indptr.device))
    idx2 = indices.reshape(n, 5).long()
    dat2 = data.reshape(n, 5)
    for d in range(5):
        hit = idx2 == cols[d][:, None]
        assert torch.equal(hit.sum(1), torch.ones(n, dtype=hit.sum(1).dtype, device=hit.device))
        want = dat2[hit]
        assert torch.equal(coef[d], want), f"direction {d}: {int((coef[d] != want).sum())} entries differ"
