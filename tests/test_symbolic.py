"""Host-side symbolic analysis (nested dissection of the periodic grid).

These tests need no GPU: the analysis is host C++ in the engine library.
A small numpy multifrontal LU (test code only) driven by the exported front
tree must reproduce the oracle's SuperLU solution, which checks the pivot
order, the boundary lists, the extend-add maps and the per-cell neighbour
maps that the GPU factor uses.
"""
import numpy as np
import pytest

from oracle import fdfd_oracle as O
from fdfdpy_gb300 import engine

OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def export_tree(sym):
    info = sym.info
    nf, n = info.n_fronts, sym.Nx * sym.Ny
    t = dict(
        p=sym.export(0, nf), m=sym.export(1, nf), parent=sym.export(2, nf), c0=sym.export(3, nf),
        c1=sym.export(4, nf), height=sym.export(5, nf), voff=sym.export(6, nf),
        level_ptr=sym.export(7, info.n_levels + 1), vars=sym.export(8, info.sum_m),
        relmap=sym.export(9, info.sum_m), nbr=sym.export(10, 4 * n).reshape(n, 4),
        vfront=sym.export(11, n), vloc=sym.export(12, n), ld=sym.export(13, nf),
        pool_off=sym.export(14, nf, np.int64))
    return t


@pytest.mark.parametrize("Nx,Ny,leaf", [(3, 3, 1), (8, 8, 4), (17, 23, 16), (40, 33, 64), (64, 64, 64),
                                        (5, 41, 8)])
def test_tree_invariants(Nx, Ny, leaf):
    sym = engine.Symbolic(Nx, Ny, leaf)
    t = export_tree(sym)
    n = Nx * Ny
    nf = sym.info.n_fronts
    # every cell is a pivot of exactly one front
    piv = np.concatenate([t["vars"][t["voff"][f]:t["voff"][f] + t["p"][f]] for f in range(nf)])
    assert np.array_equal(np.sort(piv), np.arange(n))
    assert t["parent"][-1] == -1 and t["m"][-1] == t["p"][-1]  # root: no boundary
    assert np.all(np.diff(t["height"]) >= 0)                      # level order
    for f in range(nf):
        for c in (t["c0"][f], t["c1"][f]):
            if c >= 0:
                assert t["parent"][c] == f and t["height"][c] < t["height"][f]
                rm = t["relmap"][t["voff"][c] + t["p"][c]:t["voff"][c] + t["m"][c]]
                cv = t["vars"][t["voff"][c] + t["p"][c]:t["voff"][c] + t["m"][c]]
                pv = t["vars"][t["voff"][f]:t["voff"][f] + t["m"][f]]
                assert np.array_equal(pv[rm], cv)  # extend-add map points at the same cells
    assert np.all(t["ld"] % 4 == 0) and np.all(t["ld"] >= t["m"])
    assert sym.info.pool_entries == int(np.sum(t["ld"].astype(np.int64) * t["m"]))


def multifrontal_numpy(A, t):
    """Dense multifrontal LU + solve over the exported tree (test reference)."""
    A = A.tocsr()
    nf = len(t["p"])
    fronts, upd = {}, {}
    for f in range(nf):
        p, m, vo = t["p"][f], t["m"][f], t["voff"][f]
        v = t["vars"][vo:vo + m]
        F = np.zeros((m, m), dtype=complex)
        pos = {g: k for k, g in enumerate(v)}
        for k in range(p):
            s = v[k]
            for idx in range(A.indptr[s], A.indptr[s + 1]):
                c = A.indices[idx]
                if c in pos:
                    F[k, pos[c]] += A.data[idx]
            for idx in range(A.indptr[s], A.indptr[s + 1]):  # column s, rows in the boundary
                c = A.indices[idx]
                if c in pos and pos[c] >= p:
                    F[pos[c], k] += A[c, s]
        for c in (t["c0"][f], t["c1"][f]):
            if c >= 0:
                rm = t["relmap"][t["voff"][c] + t["p"][c]:t["voff"][c] + t["m"][c]]
                F[np.ix_(rm, rm)] += upd.pop(c)
        for j in range(p):
            F[j + 1:, j] /= F[j, j]
            F[j + 1:, j + 1:] -= np.outer(F[j + 1:, j], F[j, j + 1:])
        fronts[f] = F
        upd[f] = F[p:, p:].copy()
    return fronts


def solve_numpy(fronts, t, b):
    nf = len(t["p"])
    y = b.astype(complex).copy()
    for f in range(nf):
        p, m, vo = t["p"][f], t["m"][f], t["voff"][f]
        v = t["vars"][vo:vo + m]
        F = fronts[f]
        L = np.tril(F[:p, :p], -1) + np.eye(p)
        ys = np.linalg.solve(L, y[v[:p]])
        y[v[:p]] = ys
        y[v[p:]] -= F[p:, :p] @ ys
    x = y.copy()
    for f in reversed(range(nf)):
        p, m, vo = t["p"][f], t["m"][f], t["voff"][f]
        v = t["vars"][vo:vo + m]
        F = fronts[f]
        U = np.triu(F[:p, :p])
        x[v[:p]] = np.linalg.solve(U, y[v[:p]] - F[:p, p:] @ x[v[p:]])
    return x


@pytest.mark.parametrize("Nx,Ny,leaf,pol", [(8, 8, 4, "Ez"), (17, 13, 16, "Hz"), (24, 30, 64, "Ez"),
                                            (31, 9, 8, "Hz")])
def test_numpy_multifrontal_matches_superlu(Nx, Ny, leaf, pol):
    rng = np.random.default_rng(7)
    eps = 1 + 11 * rng.random((Nx, Ny))
    dl = 0.02
    A = O.construct_A(OMEGA, Nx * dl, Ny * dl, eps, [3, 2], pol, 1e-6)
    t = export_tree(engine.Symbolic(Nx, Ny, leaf))
    fronts = multifrontal_numpy(A, t)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    x = solve_numpy(fronts, t, b)
    xr = O.solve(A, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12


def test_neighbour_maps():
    Nx, Ny = 12, 10
    sym = engine.Symbolic(Nx, Ny, 8)
    t = export_tree(sym)
    for s in range(Nx * Ny):
        f = t["vfront"][s]
        v = t["vars"][t["voff"][f]:t["voff"][f] + t["m"][f]]
        assert v[t["vloc"][s]] == s
        i, j = divmod(s, Ny)
        nbrs = [((i - 1) % Nx) * Ny + j, ((i + 1) % Nx) * Ny + j, i * Ny + (j - 1) % Ny, i * Ny + (j + 1) % Ny]
        for d, g in enumerate(nbrs):
            nl = t["nbr"][s, d]
            if nl >= 0:
                assert v[nl] == g
            else:  # eliminated earlier, in a descendant front
                fg = t["vfront"][g]
                a = fg
                while a != -1 and a != f:
                    a = t["parent"][a]
                assert a == f and fg != f


def test_flop_and_size_counts_2048():
    sym = engine.Symbolic(2048, 2048, 64)
    info = sym.info
    assert info.max_p == 4095 and info.max_m == 2047 + 4094
    # complex LU flops of the whole tree: order n^1.5 (nested dissection)
    assert 1e11 < info.factor_flops < 1e13
    assert info.pool_entries < 3e9


@pytest.mark.parametrize("Nx,Ny,leaf,B", [(8, 8, 4, 2), (17, 23, 16, 3), (40, 33, 64, 4)])
def test_batch_forest_replicates_the_tree(Nx, Ny, leaf, B):
    """The batch symbolic (one forest of B copies of the tree, for factoring B
    operators of a grid in one pass) is the single tree B times: level L
    holds the B copies of the tree's level-L fronts contiguously, copy b's
    variables are the tree's plus b n, its children / parents stay inside
    the copy, and the neighbour and extend-add maps are the tree's."""
    one = engine.Symbolic(Nx, Ny, leaf)
    fst = engine.Symbolic(Nx, Ny, leaf, batch=B)
    n = Nx * Ny
    assert fst.info.Nx == B * Nx and fst.info.Ny == Ny
    assert fst.info.n_fronts == B * one.info.n_fronts and fst.info.n_levels == one.info.n_levels
    assert fst.info.factor_flops == pytest.approx(B * one.info.factor_flops)
    nf1, nf = one.info.n_fronts, fst.info.n_fronts
    a = dict(p=one.export(0, nf1), m=one.export(1, nf1), parent=one.export(2, nf1), c0=one.export(3, nf1),
             voff=one.export(6, nf1), lp=one.export(7, one.info.n_levels + 1), vars=one.export(8, one.info.sum_m),
             relmap=one.export(9, one.info.sum_m), nbr=one.export(10, 4 * n), vfront=one.export(11, n),
             vloc=one.export(12, n))
    b = dict(p=fst.export(0, nf), m=fst.export(1, nf), parent=fst.export(2, nf), c0=fst.export(3, nf),
             voff=fst.export(6, nf), lp=fst.export(7, fst.info.n_levels + 1), vars=fst.export(8, fst.info.sum_m),
             relmap=fst.export(9, fst.info.sum_m), nbr=fst.export(10, 4 * n * B), vfront=fst.export(11, n * B),
             vloc=fst.export(12, n * B))
    assert np.array_equal(b["lp"], B * a["lp"])
    for L in range(one.info.n_levels):
        cnt = a["lp"][L + 1] - a["lp"][L]
        for copy in range(B):
            for f in range(a["lp"][L], a["lp"][L + 1]):
                g = b["lp"][L] + copy * cnt + (f - a["lp"][L])
                assert b["p"][g] == a["p"][f] and b["m"][g] == a["m"][f]
                va = a["vars"][a["voff"][f]:a["voff"][f] + a["m"][f]]
                vb = b["vars"][b["voff"][g]:b["voff"][g] + b["m"][g]]
                assert np.array_equal(vb, va + copy * n)
                assert np.array_equal(b["relmap"][b["voff"][g]:b["voff"][g] + b["m"][g]],
                                      a["relmap"][a["voff"][f]:a["voff"][f] + a["m"][f]])
                if a["parent"][f] >= 0:
                    pg = b["parent"][g]
                    assert b["lp"][L + 1] <= pg and vb[0] // n == copy
                    assert b["vars"][b["voff"][pg]] // n == copy     # the parent is in the same copy
    assert np.array_equal(b["nbr"], np.tile(a["nbr"], B))
    assert np.array_equal(b["vloc"], np.tile(a["vloc"], B))
    for copy in range(B):
        cells = np.arange(n) + copy * n
        owner = b["vfront"][cells]
        assert np.all(b["vars"][b["voff"][owner] + b["vloc"][cells]] == cells)
