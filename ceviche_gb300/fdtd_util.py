"""Host-side FDTD constants shared by the Python layer."""
import numpy as np

from .constants import C_0


def fdtd_dt(dL, stability_factor=0.5):
    """Time step of ceviche/fdtd.py:213-222 (3D Courant limit, also used in 2D)."""
    dL_sum = 3 / dL ** 2
    dL_avg = 1 / np.sqrt(dL_sum)
    return dL_avg / C_0 * stability_factor
