"""Pin the CPU oracle against golden vectors produced by the reference
itself (tests/golden/make_golden.py).  No GPU."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse.linalg as spl

from oracle import fdfd_oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_constants_bitexact():
    from fdfdpy_gb300 import constants as K
    assert K.EPSILON_0 == 8.85418782e-12 and K.MU_0 == 1.25663706e-6
    assert K.C_0 == O.C_0 and K.ETA_0 == O.ETA_0


def test_sfactors_bitexact():
    sf = np.load(GOLD / "sfactors.npz")
    for t in "abcde":
        wlen, Nw, npml, om, L0 = sf[t + "_args"]
        for s in "fb":
            assert np.array_equal(O.sfactor(wlen, L0, s, om, int(Nw), int(npml)), sf[f"{t}_{s}"])


def _cases():
    g = np.load(GOLD / "small_ops.npz")
    return g, sorted({k[:-5] for k in g.files if k.endswith("_args")})


def test_operator_and_derivs_bitexact():
    g, names = _cases()
    for nm in names:
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny, npml = int(Nx), int(Ny), [int(p0), int(p1)]
        pol = "Ez" if pol == 0 else "Hz"
        A = O.construct_A(om, Nx * dl, Ny * dl, g[nm + "_eps"], npml, pol, L0)
        assert np.array_equal(A.indptr, g[nm + "_indptr"]) and np.array_equal(A.indices, g[nm + "_indices"])
        assert np.array_equal(A.data, g[nm + "_data"]), nm
        if pol == "Hz":
            A2 = O.construct_A(om, Nx * dl, Ny * dl, g[nm + "_eps"], npml, pol, L0, averaging=False)
            assert np.array_equal(A2.data, g[nm + "_noavg_data"])
        D = O.derivs(om, Nx * dl, Ny * dl, Nx, Ny, npml, L0)
        for dn in ("Dxf", "Dxb", "Dyf", "Dyb"):
            assert np.array_equal(D[dn].data, g[f"{nm}_{dn}"]), (nm, dn)


def test_solved_fields_match_reference():
    g, names = _cases()
    for nm in names:
        if nm == "ez_12x9_L0":
            continue  # omega = 100 rad/s: a near-singular static periodic Laplacian
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny, npml = int(Nx), int(Ny), [int(p0), int(p1)]
        pol = "Ez" if pol == 0 else "Hz"
        eps = g[nm + "_eps"]
        A = O.construct_A(om, Nx * dl, Ny * dl, eps, npml, pol, L0)
        X = O.solve(A, 1j * om * g[nm + "_src"].reshape(-1))
        f = O.fields(om, Nx * dl, Ny * dl, eps, npml, pol, L0, X)
        for k, fv in zip(("_f1", "_f2", "_f3"), f):
            assert rel(fv, g[nm + k]) < 1e-12, (nm, k)
        if pol == "Hz":
            f = O.fields(om, Nx * dl, Ny * dl, eps, npml, pol, L0, X, averaging=False)
            assert rel(f[0], g[nm + "_noavg_f1"]) < 1e-12 and rel(f[1], g[nm + "_noavg_f2"]) < 1e-12


def test_ez200_point_source():
    g = np.load(GOLD / "ez200.npz")
    N = 200
    eps = np.ones((N, N))
    eps[80:120, 80:120] = 12
    A = O.construct_A(OMEGA, N * 0.02, N * 0.02, eps, [15, 15], "Ez", 1e-6)
    for r, idx, dat in zip(g["rows"], g["row_indices"], g["row_data"]):
        assert np.array_equal(A.indices[A.indptr[r]:A.indptr[r + 1]], idx)
        assert np.array_equal(A.data[A.indptr[r]:A.indptr[r + 1]], dat)
    src = np.zeros((N, N))
    src[100, 100] = 1
    X = O.solve(A, 1j * OMEGA * src.reshape(-1))
    Hx, Hy, Ez = O.fields(OMEGA, N * 0.02, N * 0.02, eps, [15, 15], "Ez", 1e-6, X)
    s = g["sample"]
    assert rel(Ez.reshape(-1)[s], g["Ez"]) < 1e-12 and rel(Hx.reshape(-1)[s], g["Hx"]) < 1e-12
    assert g["relres"] < 1e-13


def test_p_scaling_symmetrises_operator():
    """A^T = P A P^-1 with P = diag(sxf(i) syf(j)): the identity the GPU's
    transposed (adjoint) solve relies on."""
    g, names = _cases()
    for nm in names:
        Nx, Ny, p0, p1, dl, om, L0, pol = g[nm + "_args"]
        Nx, Ny, npml = int(Nx), int(Ny), [int(p0), int(p1)]
        pol = "Ez" if pol == 0 else "Hz"
        A = O.construct_A(om, Nx * dl, Ny * dl, g[nm + "_eps"], npml, pol, L0)
        P = O.p_scaling(om, L0, Nx, Ny, npml, Nx * dl, Ny * dl)
        PA = A.multiply(P[:, None]).tocsr()
        assert abs(PA - PA.T).max() <= 1e-14 * abs(PA).max(), nm


def test_adjoint_gradient_oracle_matches_finite_differences():
    rng = np.random.default_rng(11)
    Nx, Ny, dl = 20, 18, 0.02
    eps = 1 + 11 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[5, 9] = 1
    k = 14 * Ny + 9

    def J(e):
        A = O.construct_A(OMEGA, Nx * dl, Ny * dl, e, [4, 4], "Ez", 1e-6)
        E = O.solve(A, 1j * OMEGA * src.reshape(-1))
        return abs(E[k]) ** 2, A, E

    J0, A, E = J(eps)
    g = np.zeros(Nx * Ny, complex)
    g[k] = 2 * E[k]  # torch convention: grad of |E_k|^2 w.r.t. E is 2 E_k
    grad = O.adjoint_grad_eps_Ez(A, E, g, OMEGA, 1e-6)
    def Jp(p, d):
        e = eps.copy()
        e.reshape(-1)[p] += d
        return J(e)[0]

    pix = rng.choice(Nx * Ny, 8, replace=False)
    h = 1e-4
    fd = np.array([(Jp(p, h) - Jp(p, -h)) / (2 * h) for p in pix])   # central differences
    # norm-wise over the sampled pixels (weakly coupled pixels have
    # gradients far below the round-off of J itself)
    assert np.linalg.norm(fd - grad[pix]) / np.linalg.norm(grad[pix]) < 1e-6


def test_superlu_complex64_refinement_converges():
    """The premise of the mixed form: a complex64 factor refined in FP64
    reaches 1e-10 on these operators (checked on the CPU with SuperLU)."""
    g = np.load(GOLD / "hz128_blocks.npz")
    eps = g["eps"]
    A = O.construct_A(OMEGA, 1.28, 1.28, eps, [20, 20], "Hz", 1e-6).tocsc()
    b = np.zeros(128 * 128, complex)
    b[30 * 128:31 * 128] = 1j * OMEGA
    lu = spl.splu(A.astype(np.complex64))
    x = np.zeros_like(b)
    for _ in range(10):
        x = x + lu.solve((b - A @ x).astype(np.complex64)).astype(complex)
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-10
    assert rel(x, g["Hz"].reshape(-1)) < 1e-8


@pytest.mark.parametrize("tag,pol,average", [("ez", "Ez", False), ("hz", "Hz", False), ("hzy", "Hz", True)])
def test_mode_operator_and_eigenpair(tag, pol, average):
    m = np.load(GOLD / "modes.npz")
    om = 2 * np.pi * 200e12
    if tag == "hzy":
        eps = np.ones((200, 300))
        eps[90:110, :] = 12.25
        sl = eps[70:130, 20]
    else:
        eps = np.ones((600, 200))
        eps[:, 90:110] = 12.25
        sl = eps[20, 70:130]
    A1 = O.mode_operator(pol, sl, om, 0.01, 1e-6, average).toarray()
    want = m[tag + "_A1"]
    assert np.max(np.abs(A1 - want)) <= 1e-15 * np.max(np.abs(want))
    vals, vecs = O.mode_eigs(O.mode_operator(pol, sl, om, 0.01, 1e-6, average), 1, float(m[tag + "_sigma"]))
    assert abs(vals[0] - m[tag + "_eigval"][0]) <= 1e-10 * abs(vals[0])
    v, w = vecs[:, 0], m[tag + "_eigvec"][:, 0]
    assert min(np.linalg.norm(v - w), np.linalg.norm(v + w)) < 1e-8


@pytest.mark.parametrize("solver", ["newton", "born"])
def test_kerr_oracle_matches_reference(solver):
    """The oracle's Newton and Born iterations (oracle/fdfd_oracle.py) against
    the reference's solve_fields_nl on a 48 x 40 Ez grid: same iterates
    (convergence history) and the same final field."""
    g = np.load(GOLD / "kerr48.npz")
    eps, region = g["eps"], g["region"]
    Nx, Ny = eps.shape
    omega, dl, chi = float(g["omega"]), float(g["dl"]), float(g["chi"])
    src = np.zeros((Nx, Ny))
    src[10, 20] = float(g[f"{solver}_amp"])
    fn = O.newton_kerr_Ez if solver == "newton" else O.born_kerr_Ez
    E, conv = fn(omega, Nx * dl, Ny * dl, eps, [6, 6], 1e-6, src, chi / 1e-12, region, conv_threshold=1e-12,
                 max_num_iter=50 if solver == "newton" else 200)
    ref = g[f"{solver}_Ez"].reshape(-1)
    assert np.linalg.norm(E - ref) / np.linalg.norm(ref) < 1e-10
    cref = g[f"{solver}_conv"]
    cref = cref[cref > 0]
    assert len(conv) == len(cref)
    big = cref > 1e-9  # the last steps are at rounding level
    assert np.allclose(np.asarray(conv)[big], cref[big], rtol=1e-6)
