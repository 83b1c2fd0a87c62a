"""The no-allocation entry point atmo_precompute_noalloc, for callers that
cannot allocate device memory (plugins of applications that own all device
memory, latency-bound code avoiding cudaMalloc's synchronisation).  It keeps
its temporaries in a fixed device array shared by every call, so this file
checks two calls in a row against atmo_precompute through the C ABI, within
the parity tolerances of the other tests, and that oversize shapes are
refused.  It sorts last so that a run stopping at its first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

from parity import TOL_IRRADIANCE, TOL_SCATTERING, TOL_TRANSMITTANCE, check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def run(atmo, torch, fn, atm, shape, orders, combined):
    s = atmo.LutShape.of(shape)
    dev = torch.device("cuda")
    W = s.scattering_nu * s.scattering_mu_s
    T = torch.full((s.transmittance_height, s.transmittance_width, 4), -1.0, device=dev)
    S = torch.full((s.scattering_r, s.scattering_mu, W, 4), -1.0, device=dev)
    M = torch.full_like(S, -1.0)
    I = torch.full((s.irradiance_height, s.irradiance_width, 4), -1.0, device=dev)
    a = atmo.Atmosphere.from_buffer_of(atm)
    args = [C.byref(a), C.byref(s), orders, None, 0, int(combined)]
    if fn == "atmo_precompute":
        args.append(atmo.PATH_FAST)
    args += [T.data_ptr(), S.data_ptr(), None if combined else M.data_ptr(), I.data_ptr(),
             None]
    st = getattr(atmo.lib(), fn)(*args)
    assert st == 0, atmo.lib().atmo_last_error().decode()
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in (T, S, M, I)]


def same(a, b, combined):
    check("transmittance", a[0], b[0], TOL_TRANSMITTANCE)
    check("scattering", a[1], b[1], TOL_SCATTERING, channels=4 if combined else 3)
    if not combined:
        check("single_mie", a[2], b[2], TOL_SCATTERING)
    check("irradiance", a[3], b[3], TOL_IRRADIANCE)


def test_no_alloc_matches_precompute_on_two_calls_in_a_row(atmo, oracle, torch):
    earth = oracle.earth_atmosphere()
    other = oracle.earth_atmosphere(mie_g=0.7, ground_albedo=0.3)
    # Call 1: the reference's default LUT shape, combined textures.
    got = run(atmo, torch, "atmo_precompute_noalloc", earth, oracle.DEFAULT_SHAPE, 4, True)
    want = run(atmo, torch, "atmo_precompute", earth, oracle.DEFAULT_SHAPE, 4, True)
    same(got, want, True)
    # Call 2, right after, reusing the shared scratch with other parameters,
    # another shape and a separate single-Mie texture.
    got = run(atmo, torch, "atmo_precompute_noalloc", other, oracle.MEDIUM_SHAPE, 3, False)
    want = run(atmo, torch, "atmo_precompute", other, oracle.MEDIUM_SHAPE, 3, False)
    same(got, want, False)


def test_no_alloc_refuses_shapes_beyond_its_scratch(atmo, oracle, torch):
    hires = (512, 128, 64, 256, 64, 16, 128, 32)
    s = atmo.LutShape.of(hires)
    a = atmo.Atmosphere.from_buffer_of(oracle.earth_atmosphere())
    st = atmo.lib().atmo_precompute_noalloc(C.byref(a), C.byref(s), 4, None, 0, 1, 1, 1, None,
                                            1, None)
    assert st == atmo.BUDGET
    assert b"scratch" in atmo.lib().atmo_last_error()
