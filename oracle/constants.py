"""SI constants, same values as ceviche/constants.py:7-11 (test infrastructure only)."""
import numpy as np

EPSILON_0 = 8.85418782e-12
MU_0 = 1.25663706e-6
C_0 = 1 / np.sqrt(EPSILON_0 * MU_0)
ETA_0 = np.sqrt(MU_0 / EPSILON_0)
