"""LUT files in the reference's interchange format
(atmosphere/demo/webgl/precompute.cc:63-106, read by demo.js:364-377): raw
little-endian float32 RGBA texels, x fastest."""
import os

import numpy as np
import pytest

from test_capi_host import earth_model


def test_load_rejects_missing_and_missized_files(atmo, tmp_path):
    m = earth_model(atmo, shape=(64, 16, 4, 16, 8, 4, 16, 4))
    with pytest.raises(atmo.AtmoError) as e:
        m.load_luts(str(tmp_path))
    assert e.value.status == atmo.INVALID_ARG
    np.zeros(64 * 16 * 4 + 4, np.float32).tofile(tmp_path / "transmittance.dat")
    np.zeros(16 * 4 * 4, np.float32).tofile(tmp_path / "irradiance.dat")
    with pytest.raises(atmo.AtmoError) as e:
        m.load_luts(str(tmp_path))
    assert e.value.status == atmo.INVALID_ARG
    assert "bytes" in str(e.value)


def test_save_requires_init(atmo, tmp_path):
    m = earth_model(atmo)
    with pytest.raises(atmo.AtmoError) as e:
        m.save_luts(str(tmp_path))
    assert e.value.status == atmo.NOT_READY


@pytest.mark.gpu
@pytest.mark.parametrize("combined", [True, False], ids=["combined", "separate"])
def test_save_load_round_trip(atmo, torch_cuda, tmp_path, combined):
    torch = torch_cuda
    shape = (128, 32, 8, 32, 16, 8, 32, 8)
    m = earth_model(atmo, combined=combined, shape=shape)
    m.Init(4)
    m.save_luts(str(tmp_path))
    T, S, I = m.transmittance(), m.scattering(), m.irradiance()
    files = {"transmittance.dat": T, "scattering.dat": S, "irradiance.dat": I}
    if not combined:
        files["single_mie_scattering.dat"] = m.single_mie_scattering()
    for name, lut in files.items():
        raw = np.fromfile(tmp_path / name, dtype="<f4")
        assert raw.size == lut.size
        np.testing.assert_array_equal(raw, lut.ravel())
    src = (tmp_path / "atmosphere_shader.txt").read_text()
    assert src == m.shader()
    assert os.path.getsize(tmp_path / "optical_depth.dat") == T.nbytes

    fresh = earth_model(atmo, combined=combined, shape=shape)
    fresh.load_luts(str(tmp_path))
    for got, want in ((fresh.transmittance(), T), (fresh.scattering(), S),
                      (fresh.irradiance(), I)):
        np.testing.assert_array_equal(got, want)
    rng = np.random.default_rng(8)
    n = 512
    cam = np.tile([0.0, 0.0, 6361.0], (n, 1)).astype(np.float32)
    view = rng.normal(size=(n, 3))
    view = (view / np.linalg.norm(view, axis=1, keepdims=True)).astype(np.float32)
    cam_t, view_t = torch.from_numpy(cam).cuda(), torch.from_numpy(view).cuda()
    sun = torch.tensor([0.0, 0.6, 0.8], device="cuda")
    a, ta = m.lut_set().sky_radiance(cam_t, view_t, sun)
    b, tb = fresh.lut_set().sky_radiance(cam_t, view_t, sun)
    torch.testing.assert_close(a, b, rtol=0, atol=0)
    torch.testing.assert_close(ta, tb, rtol=0, atol=0)

    # Files of the reference's tool carry no optical-depth LUT: -ln T stands in.
    os.remove(tmp_path / "optical_depth.dat")
    ref_files = earth_model(atmo, combined=combined, shape=shape)
    ref_files.load_luts(str(tmp_path))
    c, tc = ref_files.lut_set().sky_radiance(cam_t, view_t, sun)
    torch.testing.assert_close(c, a, rtol=1e-5, atol=1e-12)


@pytest.mark.gpu
def test_batch_instance_save(atmo, oracle, torch_cuda, tmp_path):
    b = atmo.Batch([oracle.earth_atmosphere()], [(64, 16, 4, 16, 8, 4, 16, 4)], [2])
    b.run()
    atmo.synchronize_stream()
    b.save_luts(0, str(tmp_path))
    raw = np.fromfile(tmp_path / "scattering.dat", dtype="<f4")
    np.testing.assert_array_equal(raw, b.read(0, atmo.LUT_SCATTERING).ravel())
    assert not (tmp_path / "atmosphere_shader.txt").exists()
