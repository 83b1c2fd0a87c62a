"""The high-resolution configuration: scattering NU16 x MU_S64 x MU256 x R64
(3D 1024x256x64), transmittance 512x128, irradiance 128x32, 8 orders, Earth
with Mie g = 0.76 and ground albedo 0.3.

The FP64 oracle cannot evaluate every pass of this size in test time, so the
full-size LUTs are checked through properties that hold exactly in FP32 and
need no oracle: every pass is linear in the solar irradiance (doubling it
doubles S and I bit for bit and leaves T unchanged), every order adds a
non-negative contribution (the LUTs of 8 orders are >= those of 7, texel by
texel), and all texels are finite and non-negative.  The transmittance LUT
(every texel) and single scattering (4096 sampled texels) are compared with
the oracle directly."""
import ctypes as C

import numpy as np
import pytest

from parity import TOL_SCATTERING, TOL_TRANSMITTANCE, check

pytestmark = pytest.mark.gpu

HIRES = (512, 128, 64, 256, 64, 16, 128, 32)


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def hires_earth(oracle, solar=1.5):
    a = oracle.earth_atmosphere(mie_g=0.76, ground_albedo=0.3)
    for i in range(3):
        a.solar_irradiance[i] = solar
    return a


def run(atmo, torch, atm, orders):
    s = atmo.LutShape(*HIRES)
    T = torch.zeros((128, 512, 4), device="cuda")
    S = torch.zeros((64, 256, 1024, 4), device="cuda")
    I = torch.zeros((32, 128, 4), device="cuda")
    atmo.precompute(atm, s, orders, T, S, None, I, combined=True)
    torch.cuda.synchronize()
    return T, S, I


def test_hires_first_order_vs_oracle(atmo, oracle, torch):
    atm = hires_earth(oracle)
    T, S, _ = run(atmo, torch, atm, 1)
    L = oracle.lib()
    shp = oracle.shape(*HIRES)
    dp = oracle.dp
    nT = 512 * 128
    idx = np.arange(nT, dtype=np.int64)
    T_ref = np.zeros((nT, 4))
    L.oracle_eval_texels(0, C.byref(atm), C.byref(shp), None, None, None, None, None, None, 0,
                         nT, idx.ctypes.data_as(C.POINTER(C.c_longlong)),
                         T_ref.ctypes.data_as(dp), None, 0)
    check("hires transmittance", T.cpu().numpy().reshape(-1, 4), T_ref,
          TOL_TRANSMITTANCE, channels=3)
    # Single scattering at sampled texels, from the oracle's own transmittance.
    rng = np.random.default_rng(6)
    nS = 1024 * 256 * 64
    sidx = np.sort(rng.choice(nS, size=4096, replace=False)).astype(np.int64)
    ray, mie = np.zeros((4096, 4)), np.zeros((4096, 4))
    Tc = np.ascontiguousarray(T_ref)
    L.oracle_eval_texels(2, C.byref(atm), C.byref(shp), Tc.ctypes.data_as(dp), None, None,
                         None, None, None, 0, 4096, sidx.ctypes.data_as(C.POINTER(C.c_longlong)),
                         ray.ctypes.data_as(dp), mie.ctypes.data_as(dp), 0)
    got = S.reshape(-1, 4)[torch.from_numpy(sidx).cuda()].cpu().numpy()
    want = np.concatenate([ray[:, :3], mie[:, :1]], axis=1)   # combined: alpha = Mie red
    check("hires single scattering (sampled)", got, want, TOL_SCATTERING, channels=4)


def test_hires_eight_orders_properties(atmo, oracle, torch):
    T1, S1, I1 = run(atmo, torch, hires_earth(oracle, 1.5), 8)
    for x in (T1, S1, I1):
        assert torch.isfinite(x).all() and (x >= 0).all()
    T2, S2, I2 = run(atmo, torch, hires_earth(oracle, 3.0), 8)
    assert torch.equal(T2, T1)
    assert torch.equal(S2, 2.0 * S1)
    assert torch.equal(I2, 2.0 * I1)
    del T2, S2, I2
    _, S7, I7 = run(atmo, torch, hires_earth(oracle, 1.5), 7)
    assert (S1[..., :3] >= S7[..., :3]).all()
    assert torch.equal(S1[..., 3], S7[..., 3])   # single-Mie alpha is order 1 only
    assert (I1 >= I7).all()
    # The eighth order still adds light somewhere.
    assert (S1[..., :3] > S7[..., :3]).any()


def test_hires_eight_orders_vs_gpu_oracle(atmo, oracle, torch):
    """Every texel of the high-resolution LUTs (8 orders) against the FP64
    GPU oracle (the CPU oracle's evaluators as device code, pinned to the CPU
    oracle by tests/test_gpu_oracle.py)."""
    from parity import TOL_IRRADIANCE
    atm = hires_earth(oracle)
    T, S, I = run(atmo, torch, atm, 8)
    ref = oracle.gpu_precompute(atm, HIRES, 8, combined=True)
    check("hires transmittance", T.cpu().numpy(), ref.transmittance, TOL_TRANSMITTANCE)
    check("hires scattering", S.cpu().numpy(), ref.scattering, TOL_SCATTERING, channels=4)
    check("hires irradiance", I.cpu().numpy(), ref.irradiance, TOL_IRRADIANCE)
