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
        self._mu_r = None  # made on first read (the mu_r property)
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

    @property
    def mu_r(self):
        """Relative permeability, all ones (simulation.py:31).  The array
        is made on first read: nothing in the solve reads it, and filling
        it took about 2 ms of host time per Simulation at 2048^2."""
        if self._mu_r is None:
            self._mu_r = np.ones((self.Nx, self.Ny))
        return self._mu_r

    @mu_r.setter
    def mu_r(self, value):
        self._mu_r = value

    # ---- sources (simulation.py:45-55) ----------------------------------------
    def setup_modes(self):
        for modei in self.modes:
            modei.setup_src(self)

    def add_mode(self, neff, direction_normal, center, width, scale=1, order=1):
        self.modes.append(mode(neff, direction_normal, center, width, scale=scale, order=order))

    # ---- nonlinearity (simulation.py:57-73) -------------------------------------
    def compute_nl(self, e, matrix_format=DEFAULT_MATRIX_FORMAT):
        """eps_nl, dnl_de, dnl_deps of the field e (simulation.py:57-68),
        evaluated on the device by the Kerr kernel (fdfd_kerr_assemble);
        the attributes hold host copies, as in the reference."""
        from .nonlinear_solvers import KerrTerms
        t = KerrTerms.of(self)(e, eps_nl=True, deps=True, de=True)
        self._set_nl_device(t['eps_nl'])
        self.dnl_de, self.dnl_deps = (a.reshape(self.Nx, self.Ny) for a in engine.to_host(t['dnl_de'],
                                                                                          t['dnl_deps']))

    def _set_nl_device(self, eps_nl_dev):
        """Make a device eps_nl current (host copy in self.eps_nl)."""
        self._nl_version = getattr(self, '_nl_version', 0) + 1
        self._eps_nl_dev = (self._nl_version, eps_nl_dev.reshape(-1))
        self.eps_nl = engine.to_host(eps_nl_dev)[0].reshape(self.Nx, self.Ny)
        self._eps_nl_host_sig = (id(self.eps_nl), hash(self.eps_nl.tobytes()))

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
        self._fields_dev = {}
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

    def _eps_nl_device(self):
        """eps_nl on the device: the kernel's copy while self.eps_nl is the
        array it produced, else an upload of whatever the user assigned."""
        dev = getattr(self, '_eps_nl_dev', None)
        arr = np.ascontiguousarray(self.eps_nl, dtype=np.float64)
        sig = (id(self.eps_nl), hash(arr.tobytes()))
        if dev is not None and sig == getattr(self, '_eps_nl_host_sig', None):
            return dev[1], ('nl', dev[0])
        return engine.as_f64(arr).reshape(-1), ('nl_host',) + sig

    def _operator(self, include_nl):
        if not include_nl:
            return self._op, ('lin',)
        eps_nl, key = self._eps_nl_device()
        return self._op.with_terms(eps_add=eps_nl), key

    def solve_device(self, b, include_nl=False, precision=None, tol=None, max_iter=None, transpose=False,
                     preconditioner=None):
        """Solve A x = b on the device (b: (n,) or (nrhs, n)); returns a
        complex128 device tensor.  Reuses the cached factor.  With
        `preconditioner` (a factor of a nearby operator, e.g. the last one of
        a Kerr loop) the operator is solved by GMRES preconditioned by it and
        factored only if that does not reach the tolerance."""
        precision = precision or self.precision
        op, key = self._operator(include_nl)
        tol_ = DEFAULT_TOL[precision] if tol is None else tol
        if preconditioner is not None and (key, precision) not in self._factors:
            from . import _native
            try:
                x = preconditioner.solve(b, transpose=transpose, op=op, method='gmres', tol=tol_, max_iter=30,
                                         raise_on_fail=True)
                self.last_solve_stats = preconditioner.stats()
                return x
            except _native.NotConverged:
                pass
        fac = self._factor_for(op, key, precision)
        method = 'ir' if precision == 'c128' else self.refinement
        x = fac.solve(b, transpose=transpose, op=op, method=method,
                      tol=DEFAULT_TOL[precision] if tol is None else tol,
                      max_iter=DEFAULT_MAX_REFINE[precision] if max_iter is None else max_iter)
        self.last_solve_stats = fac.stats()
        return x

    def solve_fields(self, include_nl=False, timing=False, averaging=True, solver=DEFAULT_SOLVER,
                     matrix_format=DEFAULT_MATRIX_FORMAT, precision=None, tol=None, preconditioner=None):
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
            X = self.solve_device(b, include_nl=include_nl, precision=precision, tol=tol,
                                  preconditioner=preconditioner)
            zero_src = False
        if include_nl:
            eps_dev = self._op.eps + self._eps_nl_device()[0]
        else:
            eps_dev = self._op.eps if self.pol == 'Hz' else None
        # the primary field goes to the host while the other two are derived
        pending = None if zero_src else engine.to_host_start(X, slot=2)
        f1, f2 = self._op.fields(X, averaging=averaging, eps=eps_dev)
        F1, F2 = (a.reshape((Nx, Ny)) for a in engine.to_host(f1, f2))
        if zero_src:
            # an all-zero source gives float zeros for the primary field (linalg.py:128-129)
            F3 = np.zeros((Nx, Ny))
        else:
            F3 = engine.to_host_finish(pending).reshape((Nx, Ny))
        if timing:
            print('Linear system solve took {:.2f} seconds'.format(time() - t))
        # device copies of the fields, tied to the host arrays returned now
        names = ('Ex', 'Ey', 'Hz') if self.pol == 'Hz' else ('Hx', 'Hy', 'Ez')
        self._fields_dev[bool(include_nl)] = {nm: (d, id(h)) for nm, d, h in zip(names, (f1, f2, X), (F1, F2, F3))}
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

    # ---- flux (simulation.py:260-315): a device reduction ------------------------
    def flux_probe(self, direction_normal, center, width, nl=False):
        """Poynting flux through a line of cells normal to `direction_normal`
        (simulation.py:260-315), reduced on the device (fdfd_flux_probe)
        from the fields of the last solve (or the arrays in self.fields /
        self.fields_nl if they were set by hand).  Returns a float."""
        out = self.flux_probe_device(direction_normal, center, width, nl=nl)
        return float(out.item())

    def flux_probe_device(self, direction_normal, center, width, nl=False):
        """As flux_probe, the result left on the device (a 0-d float64
        tensor), for loops that should not synchronise."""
        from . import _native
        if direction_normal == "x":
            normal, i0, j0 = 0, int(center[0]), int(center[1] - width / 2)
            length = int(center[1] + width / 2) - j0
        elif direction_normal == "y":
            normal, i0, j0 = 1, int(center[0] - width / 2), int(center[1])
            length = int(center[0] + width / 2) - i0
        else:
            raise ValueError("The value of direction_normal is neither x nor y!")
        flds = self.fields_nl if nl else self.fields
        F, G = ('Ez', 'Hy' if normal == 0 else 'Hx') if self.pol == 'Ez' else ('Hz', 'Ey' if normal == 0 else 'Ex')
        dev = self._fields_dev.get(bool(nl), {})

        def pick(name):
            h = flds.get(name)
            d = dev.get(name)
            if d is not None and h is not None and d[1] == id(h):
                return d[0]
            if h is None:
                raise ValueError("flux_probe: field {} has not been solved".format(name))
            return engine.as_c128(h).reshape(-1)
        Fd, Gd = pick(F), pick(G)
        out = torch.empty((), dtype=torch.float64, device=Fd.device)
        if length <= 0:
            return out.zero_()
        _native.call("fdfd_flux_probe", self.Nx, self.Ny, _native.POL[self.pol], normal, i0, j0, length,
                     float(self.dl), engine._ptr(Fd), engine._ptr(Gd), engine._ptr(out), engine.stream_ptr())
        return out

    # ---- design regions (simulation.py:344-369) ---------------------------------
    def init_design_region(self, design_region, eps_m, style=''):
        """Initial permittivity of a design region (simulation.py:344-369):
        inside the region (design_region != 0) eps_r becomes eps_m ('full'),
        1 ('empty'), uniform random in [1, eps_m) from numpy's global RNG
        ('random'), or (eps_m + 1) / 2 where design_region == 1, written into
        the current eps_r array itself ('halfway'); outside it stays.  Any
        other style leaves eps_r unchanged.  Setting eps_r rebuilds the
        device operator, as the reference's setter rebuilds A."""
        region = np.asarray(design_region)
        if style == 'halfway':
            new = self.eps_r                     # the reference modifies the array in place
            new[region == 1] = eps_m / 2 + 1 / 2
        elif style in ('full', 'empty', 'random'):
            shape = self.eps_r.shape
            if style == 'full':
                new = eps_m * np.ones(shape)
            elif style == 'empty':
                new = np.ones(shape)
            else:
                new = (eps_m - 1) * np.random.random(shape) + 1
            outside = region == 0
            new[outside] = self.eps_r[outside]
        else:
            return
        self.eps_r = new

    def __deepcopy__(self, memo):
        # device handles are not deep-copyable; copy host state and rebuild
        cls = self.__class__
        new = cls.__new__(cls)
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            if k in ('_op', '_factors', '_A_host', '_derivs_host', '_fields_dev', '_eps_nl_dev'):
                continue
            setattr(new, k, deepcopy(v, memo))
        new._op = self._op
        new._factors = dict(self._factors)
        new._A_host = None
        new._derivs_host = None
        new._fields_dev = {}
        return new

    # ---- differentiable solve (no counterpart in the reference) -------------------
    def solve_fields_torch(self, eps_r=None, precision=None):
        """The three fields as torch tensors, differentiable in eps_r (a
        float64 tensor; default: the current eps_r) through the adjoint
        solve on the forward factor: (Ex, Ey, Hz) for Hz, (Hx, Hy, Ez) for
        Ez, from the current source.  With nonlinearities added (add_nl,
        Ez), the Kerr field by Newton and its adjoint."""
        from . import adjoint
        prec = precision or self.precision
        e = torch.as_tensor(np.asarray(self.eps_r) if eps_r is None else eps_r, dtype=torch.float64,
                            device=engine.device())
        src = torch.as_tensor(np.asarray(self.src), device=e.device)
        if self.nonlinearity:
            if self.pol != 'Ez':
                raise ValueError('Invalid polarization: {}'.format(str(self.pol)))
            from .nonlinear_solvers import KerrTerms  # noqa: F401  (checks the nonlinearity types)
            X = adjoint._KerrSolve.apply(e, src, self.omega, self.dl, self.NPML, self.L0, self.nonlinearity,
                                         prec, 1e-12, 50)
        else:
            X = adjoint.solve(e, src, self.omega, self.dl, self.NPML, self.pol, self.L0, prec)
        f1, f2 = adjoint.secondary_fields(X, e, self.omega, self.dl, self.NPML, self.pol, self.L0)
        return (f1, f2, X)
