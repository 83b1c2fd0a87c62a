"""The no-allocation entry point atmo_precompute_noalloc, for callers that
cannot allocate device memory (plugins of applications that own all device
memory, latency-bound code avoiding cudaMalloc's synchronisation).  It keeps
its temporaries in a fixed device array shared by every call and runs the
same kernels on the same inputs as atmo_precompute, so this file checks,
through the C ABI, that two calls in a row give LUTs bit-identical to
atmo_precompute's (the parity tolerances of the other tests would allow far
more), including the accumulating second wavelength group with a
non-identity luminance matrix; that a repeated call leaves the device's free
memory unchanged; and that oversize shapes are refused.  It sorts last so
that a run stopping at its first failure has run every other test first."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# A luminance_from_radiance-like matrix (atmosphere/model.cc:925-943 scale).
LUM = [0.71, -0.12, 0.03, -0.21, 0.93, 0.02, 0.05, -0.18, 1.12]


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def buffers(atmo, torch, shape, fill):
    s = atmo.LutShape.of(shape)
    dev = torch.device("cuda")
    W = s.scattering_nu * s.scattering_mu_s
    return [torch.full((s.transmittance_height, s.transmittance_width, 4), fill, device=dev),
            torch.full((s.scattering_r, s.scattering_mu, W, 4), fill, device=dev),
            torch.full((s.scattering_r, s.scattering_mu, W, 4), fill, device=dev),
            torch.full((s.irradiance_height, s.irradiance_width, 4), fill, device=dev)]


def call(atmo, fn, atm, shape, orders, combined, bufs, lum=None, blend=False):
    s = atmo.LutShape.of(shape)
    a = atmo.Atmosphere.from_buffer_of(atm)
    lum_arr = None if lum is None else (C.c_float * 9)(*lum)
    T, S, M, I = bufs
    args = [C.byref(a), C.byref(s), orders, lum_arr, int(blend), int(combined)]
    if fn == "atmo_precompute":
        args.append(atmo.PATH_FAST)
    args += [T.data_ptr(), S.data_ptr(), None if combined else M.data_ptr(), I.data_ptr(), None]
    st = getattr(atmo.lib(), fn)(*args)
    assert st == 0, atmo.lib().atmo_last_error().decode()


def run(atmo, torch, fn, atm, shape, orders, combined, lum=None, blend_over=None):
    """One call into fresh buffers; blend_over: an earlier group's LUTs that
    the call accumulates into (the reference's second wavelength group)."""
    bufs = buffers(atmo, torch, shape, -1.0)
    if blend_over is not None:
        for b, src in zip(bufs, blend_over):
            b.copy_(src)
    call(atmo, fn, atm, shape, orders, combined, bufs, lum, blend_over is not None)
    torch.cuda.synchronize()
    return bufs


def identical(got, want, combined):
    names = ("transmittance", "scattering", "single_mie", "irradiance")
    for name, g, w in zip(names, got, want):
        if name == "single_mie" and combined:
            continue
        assert torch_equal(g, w), "%s differs from atmo_precompute's" % name


def torch_equal(a, b):
    return bool((a == b).all().item())


def test_no_alloc_matches_precompute_on_two_calls_in_a_row(atmo, oracle, torch):
    earth = oracle.earth_atmosphere()
    other = oracle.earth_atmosphere(mie_g=0.7, ground_albedo=0.3)
    # Call 1: the reference's default LUT shape, combined textures.
    got = run(atmo, torch, "atmo_precompute_noalloc", earth, oracle.DEFAULT_SHAPE, 4, True)
    want = run(atmo, torch, "atmo_precompute", earth, oracle.DEFAULT_SHAPE, 4, True)
    identical(got, want, True)
    assert torch.isfinite(got[1]).all() and (got[1][..., :3] > 0).any()
    # Call 2, right after, reusing the shared scratch with other parameters,
    # another shape and a separate single-Mie texture.
    got = run(atmo, torch, "atmo_precompute_noalloc", other, oracle.MEDIUM_SHAPE, 3, False)
    want = run(atmo, torch, "atmo_precompute", other, oracle.MEDIUM_SHAPE, 3, False)
    identical(got, want, False)


def test_no_alloc_accumulating_group_with_luminance_matrix(atmo, oracle, torch):
    """The second wavelength group of a luminance-mode Model: the call blends
    into the first group's LUTs, through a non-identity
    luminance_from_radiance matrix (atmosphere/model.cc:1082-1083)."""
    first = run(atmo, torch, "atmo_precompute", oracle.earth_atmosphere(),
                oracle.DEFAULT_SHAPE, 4, False, lum=LUM)
    second = oracle.earth_atmosphere(mie_g=0.75, ground_albedo=0.2)
    got = run(atmo, torch, "atmo_precompute_noalloc", second, oracle.DEFAULT_SHAPE, 4, False,
              lum=LUM, blend_over=first)
    want = run(atmo, torch, "atmo_precompute", second, oracle.DEFAULT_SHAPE, 4, False,
               lum=LUM, blend_over=first)
    identical(got, want, False)
    assert not torch_equal(got[1], first[1])   # the group did accumulate


def test_no_alloc_repeated_call_leaves_free_memory_unchanged(atmo, oracle, torch):
    """After a first call (which loads the scratch array with the library's
    device code), further calls take no device memory: cudaMemGetInfo's free
    bytes are the same before and after."""
    atm = oracle.earth_atmosphere()
    bufs = buffers(atmo, torch, oracle.DEFAULT_SHAPE, 0.0)
    call(atmo, "atmo_precompute_noalloc", atm, oracle.DEFAULT_SHAPE, 4, True, bufs)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        call(atmo, "atmo_precompute_noalloc", atm, oracle.DEFAULT_SHAPE, 4, True, bufs)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_no_alloc_refuses_shapes_beyond_its_scratch(atmo, oracle, torch):
    hires = (512, 128, 64, 256, 64, 16, 128, 32)
    s = atmo.LutShape.of(hires)
    a = atmo.Atmosphere.from_buffer_of(oracle.earth_atmosphere())
    st = atmo.lib().atmo_precompute_noalloc(C.byref(a), C.byref(s), 4, None, 0, 1, 1, 1, None,
                                            1, None)
    assert st == atmo.BUDGET
    assert b"scratch" in atmo.lib().atmo_last_error()
