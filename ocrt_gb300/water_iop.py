"""Pure-seawater and CDOM inherent optical properties for the coupled solve.

The reference's water model (rt_water_iop.c) evaluates, per wavelength:
  a_w(lambda, T) = a_w(lambda, 20 C) + psi_T(lambda) (T - 20)     (rt_water_iop.c:230-250)
  b_w(lambda)    from the same table                               (rt_water_iop.c:220-224)
  a_cdom(lambda) = a440 exp(-S (lambda - 440)), b = 0             (rt_water_iop.c:411-426)
with linear interpolation in wavelength and no extrapolation: a query
outside a table is an error (rt_water_iop.c:193-211).  The tables are the
reference's own input files (inputs/water_iop/water_coef_z09_1nm.txt with
columns lambda, a_w, b_w; psi_T_rottgers2014_OCRT.txt with lambda, psi_T),
header lines ending at "/end_header", '#' comments.

This module only turns a wavelength into the (a_total, b_water) pair that
ocrt_ocean takes; the solve itself is ocrt_gb_solve_ocean.
"""
import math
import os

import numpy as np

AW_FILE = "water_coef_z09_1nm.txt"
PSI_T_FILE = "psi_T_rottgers2014_OCRT.txt"
T_REF_C = 20.0


def _read_table(path, ncol):
    rows = []
    with open(path) as fh:
        body = False
        for line in fh:
            s = line.strip()
            if not s or s.startswith("#") or s.startswith("!"):
                continue
            if s.startswith("/"):
                body = body or s.startswith("/end_header")
                continue
            parts = s.split()
            if len(parts) < ncol:
                raise ValueError(f"{path}: short data row {s!r}")
            rows.append([float(x) for x in parts[:ncol]])
            body = True
    if len(rows) < 2:
        raise ValueError(f"{path}: fewer than two rows")
    t = np.asarray(rows, dtype=np.float64)
    if np.any(np.diff(t[:, 0]) <= 0.0):
        raise ValueError(f"{path}: wavelengths not strictly increasing")
    return t


def _interp(x, y, xq, what):
    """Linear interpolation inside the table; outside it is an error."""
    if not (x[0] <= xq <= x[-1]):
        raise ValueError(f"{what}: {xq} nm outside the table [{x[0]}, {x[-1]}] nm")
    if xq == x[0]:
        return float(y[0])
    if xq == x[-1]:
        return float(y[-1])
    hi = int(np.searchsorted(x, xq, side="right"))
    lo = hi - 1
    t = (xq - x[lo]) / (x[hi] - x[lo])
    return float((1.0 - t) * y[lo] + t * y[hi])


class PureWater:
    """The pure-seawater tables of one input directory."""

    def __init__(self, directory):
        self.aw = _read_table(os.path.join(directory, AW_FILE), 3)
        p = os.path.join(directory, PSI_T_FILE)
        self.psi = _read_table(p, 2) if os.path.exists(p) else None

    def a_w(self, wl_nm, T_c=T_REF_C):
        a = _interp(self.aw[:, 0], self.aw[:, 1], wl_nm, "a_w")
        if self.psi is not None:
            a += _interp(self.psi[:, 0], self.psi[:, 1], wl_nm, "psi_T") * (T_c - T_REF_C)
        return a

    def b_w(self, wl_nm):
        return _interp(self.aw[:, 0], self.aw[:, 2], wl_nm, "b_w")

    def iops(self, wl_nm, T_c=T_REF_C, acdom440=0.0, cdom_slope=0.014):
        """(a_total, b_water) of pure seawater plus CDOM, in 1/m."""
        a, b = self.a_w(wl_nm, T_c), self.b_w(wl_nm)
        if not (a > 0.0 and b > 0.0):
            raise ValueError(f"pure-water IOPs not positive at {wl_nm} nm")
        return a + cdom_a(wl_nm, acdom440, cdom_slope), b


def cdom_a(wl_nm, a440, slope=0.014, ref_nm=440.0):
    if not (a440 > 0.0):
        return 0.0
    return max(0.0, a440 * math.exp(-slope * (wl_nm - ref_nm)))


def default_directory():
    """$OCRT_GB_WATER_IOP, else water_iop under $OCRT_GB_INPUTS (or inputs/)."""
    if os.environ.get("OCRT_GB_WATER_IOP"):
        return os.environ["OCRT_GB_WATER_IOP"]
    return os.path.join(os.environ.get("OCRT_GB_INPUTS") or "inputs", "water_iop")
