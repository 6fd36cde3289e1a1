"""Mode sources (fdfdpy/source/mode.py:9-108) on the GPU engine.

insert_mode builds the 1-D periodic slice operator on the device
(fdfd_mode_stencil), factors (A1 - sigma I) with the same multifrontal
engine (an N x 1 grid: one dense front) and runs a shift-invert subspace
iteration around sigma = (omega sqrt(mu0' eps0') neff)^2 -- the job of
ARPACK's eigs(A1, order, sigma) in the reference (mode.py:93-94,
linalg.py:110-119).  compute_normalization solves the straight-waveguide
problem through the same GPU solve (mode.py:26-60).

Eigenvectors are returned with unit 2-norm and a deterministic phase (the
largest component real and positive); ARPACK's are unit-norm with an
arbitrary sign, so a mode source agrees with the reference's up to a global
sign (flux and power do not depend on it).
"""
from copy import deepcopy

import numpy as np
import torch

from .. import engine
from ..constants import EPSILON_0, MU_0, DEFAULT_MATRIX_FORMAT


class mode:

    def __init__(self, neff, direction_normal, center, width, scale, order=1):
        self.neff = neff
        self.direction_normal = direction_normal
        self.center = center
        self.width = width
        self.order = order
        self.scale = scale

    def setup_src(self, simulation, matrix_format=DEFAULT_MATRIX_FORMAT):
        self.compute_normalization(simulation, matrix_format=matrix_format)
        self.insert_mode(simulation, simulation.src, matrix_format=matrix_format)

    def compute_normalization(self, simulation, matrix_format=DEFAULT_MATRIX_FORMAT):
        """Input power of the mode in a straight waveguide (mode.py:26-60)."""
        original_eps = simulation.eps_r
        (Nx, Ny) = original_eps.shape
        eps_max = np.max(np.abs(original_eps))
        norm_eps = np.ones((Nx, Ny))
        simulation_norm = deepcopy(simulation)
        new_center = list(self.center)
        if self.direction_normal == "x":
            inds_y = original_eps[self.center[0], :] > 1
            norm_eps[:, inds_y] = eps_max
            new_center[0] = Nx - new_center[0]
        elif self.direction_normal == "y":
            inds_x = original_eps[:, self.center[1]] > 1
            norm_eps[inds_x, :] = eps_max
            new_center[1] = Ny - new_center[1]
        else:
            raise ValueError("The value of direction_normal is not x or y!")
        simulation_norm.eps_r = norm_eps
        self.insert_mode(simulation_norm, simulation_norm.src, matrix_format=matrix_format)
        simulation_norm.solve_fields()
        W_in = simulation_norm.flux_probe(self.direction_normal, new_center, self.width)
        simulation.W_in = W_in
        # The reference reads fields['Ez'] here for both polarizations (so its
        # Hz branch fails on None); the primary field is used instead.
        prim = simulation_norm.fields['Ez'] if simulation.pol == 'Ez' else simulation_norm.fields['Hz']
        simulation.E2_in = np.sum(np.square(np.abs(prim)) * np.abs(simulation_norm.src))

    def _slice(self):
        if self.direction_normal == "x":
            inds_x = [self.center[0], self.center[0] + 1]
            inds_y = [int(self.center[1] - self.width / 2), int(self.center[1] + self.width / 2)]
        elif self.direction_normal == "y":
            inds_x = [int(self.center[0] - self.width / 2), int(self.center[0] + self.width / 2)]
            inds_y = [self.center[1], self.center[1] + 1]
        else:
            raise ValueError("The value of direction_normal is not x or y!")
        return inds_x, inds_y

    def solve_mode(self, simulation):
        """(beta^2 eigenvalue, unit eigenvector on the device) of the slice."""
        inds_x, inds_y = self._slice()
        eps_r = np.asarray(simulation.eps_r)[inds_x[0]:inds_x[1], inds_y[0]:inds_y[1]]
        EPSILON_0_ = EPSILON_0 * simulation.L0
        MU_0_ = MU_0 * simulation.L0
        est_beta = simulation.omega * np.sqrt(MU_0_ * EPSILON_0_) * self.neff
        sigma = float(np.square(est_beta))
        # grid_average(eps_slice, 'x') only averages when the slice has more
        # than one row, i.e. for a slice normal to y (mode.py:83)
        average = eps_r.shape[0] > 1
        op = engine.StencilOperator.mode_slice(simulation.pol, eps_r.reshape(-1), simulation.omega,
                                               simulation.dl, simulation.L0, sigma, average)
        vals, vecs = engine.shift_invert_eigs(op, sigma, int(self.order))
        v = vecs[:, int(self.order) - 1]
        # deterministic phase: largest component real positive
        idx = int(torch.argmax(v.abs()))
        v = v * (v[idx].abs() / v[idx])
        return vals[int(self.order) - 1], v

    def insert_mode(self, simulation, destination, matrix_format=DEFAULT_MATRIX_FORMAT):
        inds_x, inds_y = self._slice()
        _, v = self.solve_mode(simulation)
        src = v.cpu().numpy() * self.scale
        if self.direction_normal == 'x':
            src = src.reshape((1, -1))
        else:
            src = src.reshape((-1, 1))
        destination[inds_x[0]:inds_x[1], inds_y[0]:inds_y[1]] = np.abs(src) * np.sign(np.real(src))
