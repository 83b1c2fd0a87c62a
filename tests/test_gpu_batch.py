"""Batched precomputation: many atmospheres with uneven LUT shapes and order
counts in one pass sequence (CUDA graph).  Every instance must produce exactly
the LUTs it produces alone, and agree with the oracle."""
import numpy as np
import pytest

from parity import TOL_IRRADIANCE, TOL_SCATTERING, TOL_TRANSMITTANCE, check_masked, robust_masks
from test_gpu_parity import compare, compare_robust, gpu_precompute, random_atmosphere

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


SHAPES = [(64, 16, 4, 16, 8, 4, 16, 4), (128, 32, 8, 32, 16, 8, 32, 8),
          (32, 8, 2, 8, 4, 2, 8, 2), (64, 16, 6, 20, 8, 4, 16, 4)]


def test_batch_uneven_equals_alone_and_oracle(atmo, oracle, torch):
    rng = np.random.default_rng(99)
    n = 6
    atms = [random_atmosphere(oracle, rng) for _ in range(n)]
    shapes = [SHAPES[i % len(SHAPES)] for i in range(n)]
    orders = [int(rng.integers(2, 7)) for _ in range(n)]
    b = atmo.Batch(atms, shapes, orders, combined=True)
    b.run()
    atmo.synchronize_stream()
    for i in range(n):
        T = b.read(i, atmo.LUT_TRANSMITTANCE)
        S = b.read(i, atmo.LUT_SCATTERING)
        I = b.read(i, atmo.LUT_IRRADIANCE)
        alone = gpu_precompute(atmo, torch, atms[i], shapes[i], orders[i], True, 0)
        np.testing.assert_array_equal(T, alone[0])
        np.testing.assert_array_equal(S, alone[1])
        np.testing.assert_array_equal(I, alone[3])
        if i < 3:
            compare_robust(oracle, atms[i], shapes[i], orders[i], [T, S, None, I], True)


def test_mixed_shapes_batch_vs_gpu_oracle(atmo, oracle, torch):
    """The batched configuration's mix in one batch: seeded random planets at
    the half, default and double-R shapes with 2-6 orders, combined textures.
    Each member, every texel where the FP64 values are not rounding-dominated
    (masks from the FP64 GPU oracle), against the FP64 GPU oracle."""
    from precomputed_atmospheric_scattering_gb300.workloads import DEFAULT, DOUBLE_R, HALF
    rng = np.random.default_rng(2024)
    shapes = [HALF, DEFAULT, DOUBLE_R, HALF]
    orders = [5, 3, 2, 6]
    atms = [random_atmosphere(oracle, rng) for _ in shapes]
    b = atmo.Batch(atms, shapes, orders, combined=True)
    b.run()
    atmo.synchronize_stream()
    for i, (atm, shape, n) in enumerate(zip(atms, shapes, orders)):
        ref, masks = robust_masks(oracle, atm, shape, n, True, precompute=oracle.gpu_precompute)
        check_masked("transmittance", b.read(i, atmo.LUT_TRANSMITTANCE), ref.transmittance,
                     TOL_TRANSMITTANCE, masks["transmittance"])
        check_masked("scattering", b.read(i, atmo.LUT_SCATTERING), ref.scattering,
                     TOL_SCATTERING, masks["scattering"], channels=4)
        check_masked("irradiance", b.read(i, atmo.LUT_IRRADIANCE), ref.irradiance,
                     TOL_IRRADIANCE, masks["irradiance"])


def test_batch_pass_falls_back_for_every_member(atmo, oracle, torch):
    """A member whose single-scattering line exceeds the fast kernel's
    buffers (a 2048-texel transmittance row) makes the batch's
    single-scattering launch plain for every member (one launch serves them
    all); each member still matches the oracle, every texel."""
    atm = oracle.earth_atmosphere()
    shapes = [(64, 16, 4, 16, 8, 4, 16, 4), (2048, 4, 4, 16, 8, 8, 16, 4)]
    b = atmo.Batch([atm, atm], shapes, [4, 3], combined=True)
    b.run()
    atmo.synchronize_stream()
    for i, (shape, orders) in enumerate(zip(shapes, [4, 3])):
        luts = [b.read(i, atmo.LUT_TRANSMITTANCE), b.read(i, atmo.LUT_SCATTERING), None,
                b.read(i, atmo.LUT_IRRADIANCE)]
        compare(oracle.precompute(atm, shape, orders, combined=True), luts, True)


def test_batch_replay_and_parameter_update(atmo, oracle, torch):
    rng = np.random.default_rng(5)
    atms = [random_atmosphere(oracle, rng) for _ in range(3)]
    b = atmo.Batch(atms, [SHAPES[0]] * 3, [3, 4, 2])
    b.run()
    atmo.synchronize_stream()
    s0 = b.read(1, atmo.LUT_SCATTERING)
    b.run()
    atmo.synchronize_stream()
    np.testing.assert_array_equal(s0, b.read(1, atmo.LUT_SCATTERING))
    new = random_atmosphere(oracle, rng)
    new.bottom_radius, new.top_radius = atms[1].bottom_radius, atms[1].top_radius
    b.set_atmosphere(1, new)
    b.run()
    atmo.synchronize_stream()
    alone = gpu_precompute(atmo, torch, new, SHAPES[0], 4, True, 0)
    np.testing.assert_array_equal(b.read(1, atmo.LUT_SCATTERING), alone[1])
    assert b.kernel_count() > 0


def test_batch_copy_lut_is_stream_ordered(atmo, oracle, torch):
    """atmo_batch_copy_lut on a side stream, after an event of the run, gives
    the same texels as the synchronous read, into device or pinned memory."""
    b = atmo.Batch([oracle.earth_atmosphere()], [SHAPES[0]], 3)
    run_stream, copy_stream = torch.cuda.Stream(), torch.cuda.Stream()
    b.run(run_stream)
    done = torch.cuda.Event()
    done.record(run_stream)
    copy_stream.wait_event(done)
    v = b.lut_view(0, atmo.LUT_SCATTERING)
    dev = torch.empty(v.bytes // 4, device="cuda")
    pin = torch.empty(v.bytes // 4).pin_memory()
    b.copy_lut(0, atmo.LUT_SCATTERING, dev.data_ptr(), v.bytes, copy_stream)
    b.copy_lut(0, atmo.LUT_SCATTERING, pin.data_ptr(), v.bytes, copy_stream)
    copy_stream.synchronize()
    ref = b.read(0, atmo.LUT_SCATTERING).ravel()
    np.testing.assert_array_equal(dev.cpu().numpy(), ref)
    np.testing.assert_array_equal(pin.numpy(), ref)
    with pytest.raises(atmo.AtmoError):
        b.copy_lut(0, atmo.LUT_SCATTERING, dev.data_ptr(), v.bytes - 16, copy_stream)


def test_forked_graph_matches_sequential_passes(atmo, oracle, torch):
    """A batch's CUDA graph runs the indirect irradiance of order n - 1 on a
    branch beside the density pass of order n (two delta-irradiance buffers);
    time_passes launches the same passes one after another.  Every replay of
    the graph must give the sequential run's LUTs bit for bit (a race between
    the branches would show as a difference on some replay)."""
    rng = np.random.default_rng(8)
    default = (256, 64, 32, 128, 32, 8, 64, 16)
    atms = [oracle.earth_atmosphere()] + [random_atmosphere(oracle, rng) for _ in range(3)]
    shapes = [default, default, SHAPES[1], SHAPES[0]]
    b = atmo.Batch(atms, shapes, [4, 5, 3, 6])
    kinds = (atmo.LUT_TRANSMITTANCE, atmo.LUT_SCATTERING, atmo.LUT_IRRADIANCE)
    b.time_passes()
    atmo.synchronize_stream()
    want = [[b.read(i, k) for k in kinds] for i in range(len(atms))]
    for _ in range(6):
        b.run()
        atmo.synchronize_stream()
        for i in range(len(atms)):
            for k, w in zip(kinds, want[i]):
                np.testing.assert_array_equal(b.read(i, k), w)
