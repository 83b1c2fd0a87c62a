"""The checked build's device-side index checks (csrc/atmo_check.cuh).

compute-sanitizer is not available, so the library has a checked build that
tests the indices its kernels compute against the buffers they read (shared-
memory table lookups, line-build rows and taps, staged texels, the texels of
every LUT lookup), records the first failure and reads element 0 instead.
A child process loads that build (ATMO_LIBRARY=checked) and runs rebuilds
over the minimal, odd, NU-16, half, default, double-R and high-resolution
shapes on the fast and plain kernels, both texture layouts, the 15-wavelength
FP16 model, the server's rounds and shading, and the render queries and a
shading request: no check may fail, and the results must equal
the ordinary build's (the checks change no arithmetic, but the compiler
schedules the checked code differently, hence a tolerance of a few ulps).
The self-test check, which fails by construction without touching memory,
shows that the record works.  Nothing here makes an invalid access.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checked_run(tmp_path_factory, atmo):
    path = str(tmp_path_factory.mktemp("checks") / "checked.npz")
    env = dict(os.environ, ATMO_LIBRARY="checked")
    r = subprocess.run([sys.executable, os.path.join(HERE, "device_checks_child.py"), path],
                       env=env, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return dict(np.load(path))


def test_checked_build_records_no_failure(checked_run):
    compiled, _ = checked_run["record"]
    assert compiled == 1, "the child did not load the checked build"
    assert str(checked_run["failure"]) == "None", "a device check failed: %s" % checked_run["failure"]


def test_checked_build_selftest_is_recorded_and_reset(checked_run):
    assert str(checked_run["selftest"]) == "('self-test', 5)"
    assert str(checked_run["after_reset"]) == "None"


def test_checked_build_matches_the_ordinary_build(checked_run, atmo):
    sys.path.insert(0, HERE)
    from device_checks_child import run_workloads
    ordinary = run_workloads(atmo)
    for k, want in ordinary.items():
        got = checked_run[k]
        assert got.shape == want.shape, k
        scale = np.maximum(np.abs(want), 1e-6 * np.abs(want).max() + 1e-30)
        err = float(np.max(np.abs(got - want) / scale))
        # The FP16 model's LUTs ("m*"): one FP16 ulp if an FP32 value rounds
        # the other way.
        tol = 2.0 ** -10 if k.startswith("m") else 1e-5
        assert err <= tol, "%s differs from the ordinary build by %g" % (k, err)


def test_ordinary_build_has_no_checks(atmo):
    compiled, failure = atmo.device_checks()
    assert not compiled and failure is None
    atmo.device_checks_selftest()
    atmo.synchronize_stream()
    assert atmo.device_checks() == (False, None)
