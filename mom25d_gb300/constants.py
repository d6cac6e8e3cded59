"""Physical constants and unit helpers (SI), as in mom25d/constants.py:1-6."""

import math

C0 = 299792458.0
MU0 = 4e-7 * math.pi
EPS0 = 1.0 / (MU0 * C0 ** 2)
ETA0 = MU0 * C0

mm = 1e-3
um = 1e-6
GHz = 1e9
MHz = 1e6
