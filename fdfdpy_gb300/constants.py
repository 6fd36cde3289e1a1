"""Physical constants and defaults, bit-identical to fdfdpy/constants.py:1-10."""
from numpy import sqrt

EPSILON_0 = 8.85418782e-12
MU_0 = 1.25663706e-6
C_0 = sqrt(1 / EPSILON_0 / MU_0)
ETA_0 = sqrt(MU_0 / EPSILON_0)

DEFAULT_MATRIX_FORMAT = 'csr'
DEFAULT_SOLVER = 'pardiso'
DEFAULT_LENGTH_SCALE = 1e-6  # microns

# Engine defaults (no counterpart in the reference).
DEFAULT_PRECISION = 'c128'   # the plain drop-in: complex128 factor
DEFAULT_LEAF_AREA = 64       # nested-dissection leaf size (cells)
DEFAULT_TOL = {'c128': 1e-12, 'c64': 1e-10, 'c64tc': 1e-10}
DEFAULT_MAX_REFINE = {'c128': 5, 'c64': 30, 'c64tc': 30}
