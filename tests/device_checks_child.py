"""Workloads of the device-check test (tests/test_gpu_device_checks.py).

run_workloads(atmo) runs, through the package's public API, rebuilds that
reach every kernel and index path of the precomputation -- a combined batch of
uneven shapes (the minimal and an odd shape, NU 16 with a wide irradiance LUT,
the half, default and double-R shapes, 2 to 5 orders), a separate-texture
batch, the plain kernels, the 15-wavelength FP16 model, the server's rounds
and shading, the high-resolution shape (4 line columns per thread, rows in the
order of their rays' invariant) and the render queries and a shading request
-- and returns their outputs as host arrays.

Run as a script with ATMO_LIBRARY=checked, it loads the checked build of the
library, runs the workloads, reads the check record, then launches the
self-test check and reads the record again, and saves everything to the .npz
named on the command line; the test compares the LUTs with the ordinary
build's.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

COMBINED = [((2, 2, 2, 4, 2, 2, 2, 2), 2), ((33, 9, 5, 14, 5, 3, 17, 5), 3),
            ((64, 16, 4, 16, 8, 16, 256, 4), 4), ((128, 32, 16, 64, 16, 4, 32, 8), 5),
            ((256, 64, 32, 128, 32, 8, 64, 16), 4), ((256, 64, 64, 128, 32, 8, 64, 16), 3)]
SEPARATE = [((64, 16, 4, 16, 8, 4, 16, 4), 4), ((128, 32, 8, 32, 16, 8, 32, 8), 3)]
PLAIN_SHAPE = (64, 16, 4, 16, 8, 4, 16, 4)
HIRES = (512, 128, 64, 256, 64, 16, 128, 32)


def run_workloads(atmo):
    import torch
    from precomputed_atmospheric_scattering_gb300 import workloads as W

    out = {}
    rng = np.random.default_rng(5)
    kinds = {"T": atmo.LUT_TRANSMITTANCE, "S": atmo.LUT_SCATTERING, "I": atmo.LUT_IRRADIANCE}

    def read_batch(tag, b, n, single_mie=False):
        for i in range(n):
            for k, kind in kinds.items():
                out["%s%d%s" % (tag, i, k)] = b.read(i, kind)
            if single_mie:
                out["%s%dM" % (tag, i)] = b.read(i, atmo.LUT_SINGLE_MIE)

    atms = [W.random_rebuild(rng)[0] for _ in COMBINED]
    atms[4] = W.earth()   # the default-shape set that the queries below use
    b = atmo.Batch(atms, [s for s, _ in COMBINED], [o for _, o in COMBINED])
    b.run()
    atmo.synchronize_stream()
    read_batch("c", b, len(COMBINED))
    # Render queries and a shading request on the default-shape set.
    lut = b.lut_set(4)
    dev = torch.device("cuda")
    n = 4096
    cam = torch.from_numpy(np.tile([0.0, 0.0, 6361.0], (n, 1)).astype(np.float32)).to(dev)
    ray = torch.from_numpy(rng.normal(size=(n, 3)).astype(np.float32)).to(dev)
    ray = ray / ray.norm(dim=1, keepdim=True)
    sun = torch.tensor([0.0, 0.6, 0.8], device=dev)
    sky, tr = lut.sky_radiance(cam, ray, sun)
    pt = cam + ray * torch.from_numpy(rng.uniform(0.1, 50.0, (n, 1)).astype(np.float32)).to(dev)
    to_pt, tr_pt = lut.sky_radiance_to_point(cam, pt, sun)
    irr_sun, irr_sky = lut.sun_and_sky_irradiance(pt, ray, sun)
    view = W.random_view(rng, 6360.0, width=192, height=108)
    depth = torch.from_numpy(rng.uniform(0.1, 100.0, 192 * 108).astype(np.float32)).to(dev)
    shade_sky, shaded = lut.shade_view(view, depth)
    torch.cuda.synchronize()
    for k, v in (("q_sky", sky), ("q_tr", tr), ("q_to_pt", to_pt), ("q_tr_pt", tr_pt),
                 ("q_irr_sun", irr_sun), ("q_irr_sky", irr_sky), ("q_shade_sky", shade_sky),
                 ("q_shaded", shaded)):
        out[k] = v.cpu().numpy()
    del lut, b

    b = atmo.Batch([W.earth(mie_g=0.7, albedo=0.3)] * len(SEPARATE), [s for s, _ in SEPARATE],
                   [o for _, o in SEPARATE], combined=False)
    b.run()
    atmo.synchronize_stream()
    read_batch("s", b, len(SEPARATE), single_mie=True)
    del b

    s = atmo.LutShape.of(PLAIN_SHAPE)
    T = torch.zeros((s.transmittance_height, s.transmittance_width, 4), device=dev)
    S = torch.zeros((s.scattering_r, s.scattering_mu, s.scattering_nu * s.scattering_mu_s, 4),
                    device=dev)
    I = torch.zeros((s.irradiance_height, s.irradiance_width, 4), device=dev)
    atmo.precompute(W.earth(), PLAIN_SHAPE, 4, T, S, None, I, path=atmo.PATH_PLAIN)
    torch.cuda.synchronize()
    out["pT"], out["pS"], out["pI"] = T.cpu().numpy(), S.cpu().numpy(), I.cpu().numpy()

    # The 15-wavelength FP16 model (5 wavelength groups blending into the same
    # LUTs, the luminance matrices, the transmittance recomputed, FP16 output).
    m = W.spectral_earth_model(PLAIN_SHAPE)
    m.Init(4)
    out["mT"], out["mS"] = m.transmittance(), m.scattering()
    out["mM"], out["mI"] = m.single_mie_scattering(), m.irradiance()
    del m

    # The server: pool-carved instances, rebuilds of two shapes built in
    # rounds beside each other, then a shading request on one of them.
    srv = atmo.Server()
    ids = [srv.submit_rebuild(W.earth(), PLAIN_SHAPE, 3),
           srv.submit_rebuild(W.earth(mie_g=0.7), (128, 32, 8, 32, 16, 8, 32, 8), 4)]
    for t in ids:
        srv.wait(t)
    view = W.random_view(rng, 6360.0, width=96, height=54)
    depth = torch.from_numpy(rng.uniform(0.1, 100.0, 96 * 54).astype(np.float32)).to(dev)
    sky_t = torch.empty((54, 96, 4), device=dev)
    shaded_t = torch.empty_like(sky_t)
    srv.wait(srv.submit_shade(ids[1], view, depth, sky_t, shaded_t))
    for j, t in enumerate(ids):
        lut = srv.lut_set(t)
        for k, kind in kinds.items():
            out["v%d%s" % (j, k)] = lut.read(kind)
        del lut
    out["v_sky"], out["v_shaded"] = sky_t.cpu().numpy(), shaded_t.cpu().numpy()
    srv.close()

    b = atmo.Batch([W.hires_earth()], [HIRES], 3)
    b.run()
    atmo.synchronize_stream()
    out["hS"] = b.read(0, atmo.LUT_SCATTERING)[::7, ::5]
    out["hI"] = b.read(0, atmo.LUT_IRRADIANCE)
    del b
    return out


def main(path):
    sys.path.insert(0, ROOT)
    import precomputed_atmospheric_scattering_gb300 as atmo

    assert atmo.CHECKED, "run with ATMO_LIBRARY=checked"
    atmo.build()
    atmo.lib()
    atmo.device_checks(reset=True)
    out = run_workloads(atmo)
    compiled, failure = atmo.device_checks(reset=True)
    atmo.device_checks_selftest()
    _, selftest = atmo.device_checks(reset=True)
    _, after_reset = atmo.device_checks()
    out["record"] = np.array([int(compiled), -1 if failure is None else 0], np.int64)
    out["failure"] = np.array(str(failure))
    out["selftest"] = np.array(str(selftest))
    out["after_reset"] = np.array(str(after_reset))
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
