"""``Simulation``: the drop-in counterpart of fdfdpy/simulation.py:15-436.

Same constructor, attributes and methods; the operator lives on the GPU
(assembled and factored there), ``A``/``derivs`` are materialised as host
scipy CSR copies only when read, and the factor of the current operator is
kept on the device and reused while only the source changes.
"""
from __future__ import annotations

from copy import deepcopy

import numpy as np
import torch

from . import engine
from .constants import (DEFAULT_LENGTH_SCALE, DEFAULT_MATRIX_FORMAT, DEFAULT_SOLVER, EPSILON_0,
                        MU_0, DEFAULT_PRECISION, DEFAULT_TOL, DEFAULT_MAX_REFINE)
from .linalg import grid_average
from .nonlinearity import Nonlinearity
from .source.mode import mode

_FIELD_NAMES = ['Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz']


class Simulation:

    def __init__(self, omega, eps_r, dl, NPML, pol, L0=DEFAULT_LENGTH_SCALE):
        self.L0 = L0
        self.omega = float(omega)
        self.dl = float(dl)
        self.NPML = [int(n) for n in NPML]
        self.pol = pol
        self._check_inputs()

        (Nx, Ny) = eps_r.shape
        self.Nx = Nx
        self.Ny = Ny
        self.mu_r = np.ones((self.Nx, self.Ny))
        self.src = np.zeros((self.Nx, self.Ny))
        self.xrange = [0, float(Nx * self.dl)]
        self.yrange = [0, float(Ny * self.dl)]
        self.precision = DEFAULT_PRECISION
        # refinement of mixed-precision solves: 'gmres' (factor-preconditioned
        # GMRES) or 'ir' (plain iterative refinement); complex128 uses 'ir'
        self.refinement = 'ir'
        self.last_solve_stats = None

        self.eps_r = eps_r

        self.modes = []
        self.nonlinearity = []
        self.eps_nl = np.zeros(eps_r.shape)
        self.dnl_de = np.zeros(eps_r.shape)
        self.dnl_deps = np.zeros(eps_r.shape)

    # ---- sources (simulation.py:45-55) ----------------------------------------
    def setup_modes(self):
        for modei in self.modes:
            modei.setup_src(self)

    def add_mode(self, neff, direction_normal, center, width, scale=1, order=1):
        self.modes.append(mode(neff, direction_normal, center, width, scale=scale, order=order))

    # ---- nonlinearity (simulation.py:57-73) -------------------------------------
    def compute_nl(self, e, matrix_format=DEFAULT_MATRIX_FORMAT):
        self.eps_nl = np.zeros(self.eps_r.shape)
        self.dnl_de = np.zeros(self.eps_r.shape)
        self.dnl_deps = np.zeros(self.eps_r.shape)
        for nli in self.nonlinearity:
            self.eps_nl = self.eps_nl + nli.eps_nl(e, self.eps_r)
            self.dnl_de = self.dnl_de + nli.dnl_de(e, self.eps_r)
            self.dnl_deps = self.dnl_deps + nli.dnl_deps(e, self.eps_r)
        self._nl_version = getattr(self, '_nl_version', 0) + 1

    @property
    def Anl(self):
        import scipy.sparse as sp
        Nbig = self.Nx * self.Ny
        return sp.spdiags(self.omega ** 2 * EPSILON_0 * self.L0 * np.asarray(self.eps_nl).reshape((-1,)),
                          0, Nbig, Nbig, format=DEFAULT_MATRIX_FORMAT)

    def add_nl(self, chi, nl_region, nl_type='kerr', eps_scale=False, eps_max=None):
        self.nonlinearity.append(Nonlinearity(chi / np.square(self.L0), nl_region, nl_type, eps_scale, eps_max))

    # ---- permittivity (simulation.py:75-101) -----------------------------------
    @property
    def eps_r(self):
        return self.__eps_r

    @eps_r.setter
    def eps_r(self, new_eps):
        self.__eps_r = new_eps
        self._op = engine.DeviceOperator(self.omega, new_eps, self.xrange[1] - self.xrange[0],
                                         self.yrange[1] - self.yrange[0], self.NPML, self.pol, self.L0)
        self._A_host = None
        self._derivs_host = None
        self._factors = {}
        self.fields = {f: None for f in _FIELD_NAMES}
        self.fields_nl = {f: None for f in _FIELD_NAMES}

    def reset_eps(self, new_eps):
        self.eps_r = new_eps

    @property
    def A(self):
        """The operator as a host scipy CSR matrix (materialised on demand)."""
        if self._A_host is None:
            A = self._op.csr()
            A.fdfd_operator = self._op
            self._A_host = A
        return self._A_host

    @property
    def derivs(self):
        if self._derivs_host is None:
            self._derivs_host = {k: self._op.deriv_csr(k) for k in ('Dyb', 'Dxb', 'Dxf', 'Dyf')}
        return self._derivs_host

    def compute_index_shift(self):
        _ = self.solve_fields()
        _ = self.solve_fields_nl()
        index_nl = np.sqrt(np.real(self.eps_r + self.eps_nl))
        index_lin = np.sqrt(np.real(self.eps_r))
        return np.abs(index_nl - index_lin)

    # ---- solve (simulation.py:112-178) -----------------------------------------
    def _factor_for(self, op, key, precision):
        fac = self._factors.get((key, precision))
        if fac is None:
            # one cached factor per operator state and precision
            self._factors = {k: v for k, v in self._factors.items() if k[0] == key}
            fac = engine.Factor(engine.symbolic_for(self.Nx, self.Ny), precision).numeric(op)
            self._factors[(key, precision)] = fac
        return fac

    def _operator(self, include_nl):
        if not include_nl:
            return self._op, ('lin',)
        return (self._op.with_terms(eps_add=np.asarray(self.eps_nl, dtype=np.float64)),
                ('nl', getattr(self, '_nl_version', 0)))

    def solve_device(self, b, include_nl=False, precision=None, tol=None, max_iter=None, transpose=False):
        """Solve A x = b on the device (b: (n,) or (nrhs, n)); returns a
        complex128 device tensor.  Reuses the cached factor."""
        precision = precision or self.precision
        op, key = self._operator(include_nl)
        fac = self._factor_for(op, key, precision)
        method = 'ir' if precision == 'c128' else self.refinement
        x = fac.solve(b, transpose=transpose, op=op, method=method,
                      tol=DEFAULT_TOL[precision] if tol is None else tol,
                      max_iter=DEFAULT_MAX_REFINE[precision] if max_iter is None else max_iter)
        self.last_solve_stats = fac.stats()
        return x

    def solve_fields(self, include_nl=False, timing=False, averaging=True, solver=DEFAULT_SOLVER,
                     matrix_format=DEFAULT_MATRIX_FORMAT, precision=None, tol=None):
        if solver.lower() not in ('pardiso', 'scipy'):
            raise ValueError('Invalid solver choice: {}, options are pardiso or scipy'.format(str(solver)))
        if self.pol not in ('Ez', 'Hz'):
            raise ValueError('Invalid polarization: {}'.format(str(self.pol)))
        from time import time
        t = time()
        (Nx, Ny) = self.src.shape
        # b = 1j * omega * src, formed on the device from the uploaded source
        src = np.asarray(self.src)
        src_dev = engine.as_f64(src) if not np.iscomplexobj(src) else engine.as_c128(src)
        b = (src_dev.reshape(-1).to(torch.complex128) * (1j * self.omega)).contiguous()
        if not bool(torch.any(src_dev != 0)):
            X = torch.zeros(Nx * Ny, dtype=torch.complex128, device=engine.device())
            zero_src = True
        else:
            X = self.solve_device(b, include_nl=include_nl, precision=precision, tol=tol)
            zero_src = False
        if include_nl:
            eps_dev = engine.as_f64(self.eps_r + self.eps_nl).reshape(-1)
        else:
            eps_dev = self._op.eps if self.pol == 'Hz' else None
        f1, f2 = self._op.fields(X, averaging=averaging, eps=eps_dev)
        if zero_src:
            # an all-zero source gives float zeros for the primary field (linalg.py:128-129)
            F1, F2 = (a.reshape((Nx, Ny)) for a in engine.to_host(f1, f2))
            F3 = np.zeros((Nx, Ny))
        else:
            F1, F2, F3 = (a.reshape((Nx, Ny)) for a in engine.to_host(f1, f2, X))
        if timing:
            print('Linear system solve took {:.2f} seconds'.format(time() - t))
        if self.pol == 'Hz':
            if not include_nl:
                self.fields['Ex'], self.fields['Ey'], self.fields['Hz'] = F1, F2, F3
            return (F1, F2, F3)
        if not include_nl:
            self.fields['Hx'], self.fields['Hy'], self.fields['Ez'] = F1, F2, F3
        return (F1, F2, F3)

    def solve_fields_nl(self, timing=False, averaging=True, Estart=None, solver_nl='newton',
                        conv_threshold=1e-10, max_num_iter=50, solver=DEFAULT_SOLVER,
                        matrix_format=DEFAULT_MATRIX_FORMAT):
        from .nonlinear_solvers import born_solve, newton_solve
        if self.pol not in ('Ez', 'Hz'):
            raise ValueError('Invalid polarization: {}'.format(str(self.pol)))
        if solver_nl == 'born':
            out = born_solve(self, Estart, conv_threshold, max_num_iter, averaging=averaging)
        elif solver_nl == 'newton':
            out = newton_solve(self, Estart, conv_threshold, max_num_iter, averaging=averaging)
        else:
            raise AssertionError("solver must be one of {'born', 'newton'}")
        names = ('Hx', 'Hy', 'Ez') if self.pol == 'Ez' else ('Ex', 'Ey', 'Hz')
        for nm, v in zip(names, out[:3]):
            self.fields_nl[nm] = v
        return out

    def _check_inputs(self):
        assert self.L0 > 0, "L0 must be a positive number, was supplied {},".format(str(self.L0))
        assert len(self.NPML) == 2, "yrange must be a list of length 2, was supplied {}, which is of length {}".format(str(self.NPML), len(self.NPML))
        assert self.NPML[0] >= 0 and self.NPML[1] >= 0, "both elements of NPML must be >= 0"
        assert self.pol in ['Ez', 'Hz'], "pol must be one of 'Ez' or 'Hz'"

    # ---- flux (simulation.py:260-315), host reduction on a line -----------------
    def flux_probe(self, direction_normal, center, width, nl=False):
        if direction_normal == "x":
            inds_x = [center[0], center[0] + 1]
            inds_y = [int(center[1] - width / 2), int(center[1] + width / 2)]
        elif direction_normal == "y":
            inds_x = [int(center[0] - width / 2), int(center[0] + width / 2)]
            inds_y = [center[1], center[1] + 1]
        else:
            raise ValueError("The value of direction_normal is neither x nor y!")
        flds = self.fields_nl if nl else self.fields
        sx = slice(inds_x[0], inds_x[1] + 1)
        sy = slice(inds_y[0], inds_y[1] + 1)
        cx = slice(inds_x[0], inds_x[1])
        cy = slice(inds_y[0], inds_y[1])
        if self.pol == 'Ez':
            Ez, Hx, Hy = flds['Ez'], flds['Hx'], flds['Hy']
            if direction_normal == "x":
                Ez_x = grid_average(Ez[sx, sy], 'x')[:-1, :-1]
                return self.dl * np.sum(-1 / 2 * np.real(Ez_x * np.conj(Hy[cx, cy])))
            Ez_y = grid_average(Ez[sx, sy], 'y')[:-1, :-1]
            return self.dl * np.sum(1 / 2 * np.real(Ez_y * np.conj(Hx[cx, cy])))
        Hz, Ex, Ey = flds['Hz'], flds['Ex'], flds['Ey']
        if direction_normal == "x":
            Hz_x = grid_average(Hz[sx, sy], 'x')[:-1, :-1]
            return self.dl * np.sum(1 / 2 * np.real(Ey[cx, cy] * np.conj(Hz_x)))
        Hz_y = grid_average(Hz[sx, sy], 'y')[:-1, :-1]
        return self.dl * np.sum(-1 / 2 * np.real(Ex[cx, cy] * np.conj(Hz_y)))

    # ---- design regions (simulation.py:344-369) ---------------------------------
    def init_design_region(self, design_region, eps_m, style=''):
        if style == 'full':
            eps_full = eps_m * np.ones(self.eps_r.shape)
            eps_full[design_region == 0] = self.eps_r[design_region == 0]
            self.eps_r = eps_full
        elif style == 'halfway':
            eps_halfway = self.eps_r
            eps_halfway[design_region == 1] = eps_m / 2 + 1 / 2
            self.eps_r = eps_halfway
        elif style == 'empty':
            eps_empty = np.ones(self.eps_r.shape)
            eps_empty[design_region == 0] = self.eps_r[design_region == 0]
            self.eps_r = eps_empty
        elif style == 'random':
            eps_random = (eps_m - 1) * np.random.random(self.eps_r.shape) + 1
            eps_random[design_region == 0] = self.eps_r[design_region == 0]
            self.eps_r = eps_random

    def __deepcopy__(self, memo):
        # device handles are not deep-copyable; copy host state and rebuild
        cls = self.__class__
        new = cls.__new__(cls)
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            if k in ('_op', '_factors', '_A_host', '_derivs_host'):
                continue
            setattr(new, k, deepcopy(v, memo))
        new._op = self._op
        new._factors = dict(self._factors)
        new._A_host = None
        new._derivs_host = None
        return new
