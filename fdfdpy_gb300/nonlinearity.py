"""Kerr nonlinearity terms (fdfdpy/nonlinearity.py:6-37).

eps_nl(e)   = 3 chi region |e|^2 [(eps - 1)/(eps_max - 1) if eps_scale]
dnl_de(e)   = 3 chi region conj(e) [...]
dnl_deps(e) = 3 chi region |e|^2 / (eps_max - 1)  (0 without eps_scale)
``chi`` arrives already divided by L0^2 (simulation.add_nl).
"""
import numpy as np


class Nonlinearity:

    def __init__(self, chi, nl_region, nl_type='kerr', eps_scale=False, eps_max=None):
        self.chi = chi
        self.nl_region = nl_region
        self.nl_type = nl_type
        self.eps_scale = eps_scale
        self.eps_max = eps_max
        if nl_type != 'kerr':
            raise AssertionError("Only 'kerr' type nonlinearity is supported")
        if eps_scale:
            if eps_max is None:
                raise AssertionError("Must provide eps_max when eps_scale is True")
            self.eps_nl = lambda e, eps_r: 3 * chi * nl_region * np.square(np.abs(e)) * ((eps_r - 1) / (eps_max - 1))
            self.dnl_de = lambda e, eps_r: 3 * chi * nl_region * np.conj(e) * ((eps_r - 1) / (eps_max - 1))
            self.dnl_deps = lambda e, eps_r: 3 * chi * nl_region * np.square(np.abs(e)) * (1 / (eps_max - 1))
        else:
            self.eps_nl = lambda e, eps_r: 3 * chi * nl_region * np.square(np.abs(e))
            self.dnl_de = lambda e, eps_r: 3 * chi * nl_region * np.conj(e)
            self.dnl_deps = lambda e, eps_r: 0
