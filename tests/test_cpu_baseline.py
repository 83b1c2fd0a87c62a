"""The CPU baseline's timing leg (bench.py: the FP64 oracle on the host cores):
both work partitions -- 64-texel blocks, and the reference CPU driver's rows and
r-slices (atmosphere/reference/model.cc:140-237) -- run every pass, and a
sampled run (density and multiple scattering on every stride-th texel) times
those passes in proportion."""
import ctypes as C

import numpy as np
import pytest


def timed(O, shp, stride, by_rows, threads=4):
    atm = O.earth_atmosphere()
    sec = np.zeros(6)
    rc = O.lib().oracle_time_precompute_partitioned(C.byref(atm), C.byref(shp), 3, stride,
                                                    threads, int(by_rows), O._arr(sec))
    assert rc == 0
    return sec


@pytest.mark.parametrize("by_rows", [False, True], ids=["blocks", "reference_rows"])
def test_every_pass_is_timed(oracle, by_rows):
    shp = oracle.shape(*oracle.SMALL_SHAPE)
    sec = timed(oracle, shp, 1, by_rows)
    assert np.all(sec > 0.0), sec


def test_sampled_passes_scale(oracle):
    """Density on every 8th texel takes about 1/8 of the full pass (loosely:
    the host is shared with other work)."""
    shp = oracle.shape(*oracle.SMALL_SHAPE)
    full = min(timed(oracle, shp, 1, False)[3] for _ in range(2))
    sampled = min(timed(oracle, shp, 8, False)[3] for _ in range(2))
    assert sampled < 0.5 * full, (sampled, full)
