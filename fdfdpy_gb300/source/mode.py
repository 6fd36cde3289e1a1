"""Mode sources (fdfdpy/source/mode.py:9-108)."""
import numpy as np


class mode:

    def __init__(self, neff, direction_normal, center, width, scale, order=1):
        self.neff = neff
        self.direction_normal = direction_normal
        self.center = center
        self.width = width
        self.order = order
        self.scale = scale

    def setup_src(self, simulation, matrix_format='csr'):
        raise NotImplementedError("mode sources are not available yet")
