"""Parity metric shared by the GPU tests.

Per-texel relative error of a GPU LUT against the FP64 oracle:
    err = |gpu - oracle| / max(|oracle|, FLOOR * max|oracle of that channel|)
with FLOOR = 1e-6 so that texels that are exactly or nearly zero (sun far
below the horizon, no scattering) are compared in absolute terms at one
millionth of the LUT's range.  The bars: TOL_TRANSMITTANCE = 1e-4 and
TOL_SCATTERING = TOL_IRRADIANCE = 1e-3 (the tolerances the build targets).
"""
import numpy as np

FLOOR = 1e-6
TOL_TRANSMITTANCE = 1e-4
TOL_SCATTERING = 1e-3
TOL_IRRADIANCE = 1e-3


def rel_err(gpu, ref, channels=3, floor=FLOOR):
    g = np.asarray(gpu, np.float64)[..., :channels].reshape(-1, channels)
    r = np.asarray(ref, np.float64)[..., :channels].reshape(-1, channels)
    scale = np.abs(r).max(axis=0)
    scale = np.where(scale > 0, scale, 1.0)
    den = np.maximum(np.abs(r), floor * scale)
    e = np.abs(g - r) / den
    return float(e.max()), float(np.percentile(e, 99))


def check(name, gpu, ref, tol, channels=3, report=None):
    mx, p99 = rel_err(gpu, ref, channels)
    if report is not None:
        report[name] = (mx, p99)
    assert mx <= tol, "%s: max relative error %.3g > %.3g (p99 %.3g)" % (name, mx, tol, p99)
    return mx
