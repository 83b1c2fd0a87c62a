"""The autotuner of the row-restructured kernels: tunings are checked for
launchability on the host, registered per LUT shape, and never change a
result (bit-identical LUTs under every block shape)."""
import numpy as np
import pytest

SMALL = (64, 16, 4, 16, 8, 4, 16, 4)
MEDIUM = (128, 32, 8, 32, 16, 8, 32, 8)


def test_set_and_get_tuning(atmo):
    t = atmo.Tuning(2, 3, 4, 1)
    atmo.set_tuning(SMALL, t)            # W = 32: up to 4 rows of 32 texels per block
    got = atmo.get_tuning(SMALL)
    assert (got.multiple_rows, got.multiple_group, got.single_rows, got.single_group) == \
        (2, 3, 4, 1)
    atmo.set_tuning(SMALL, None)
    got = atmo.get_tuning(SMALL)
    assert (got.multiple_rows, got.multiple_group, got.single_rows, got.single_group) == \
        (0, 0, 0, 0)


@pytest.mark.parametrize("bad", [(2, 1, 0, 0), (1, 9, 0, 0), (0, 0, 5, 1), (1, 0, 0, 0)])
def test_unlaunchable_tunings_are_rejected(atmo, bad):
    # The default shape's rows are 256 texels wide: one row per block only.
    with pytest.raises(atmo.AtmoError) as e:
        atmo.set_tuning(atmo.DEFAULT_SHAPE, atmo.Tuning(*bad))
    assert e.value.status == atmo.INVALID_ARG
    assert atmo.get_tuning(atmo.DEFAULT_SHAPE).multiple_rows == 0


@pytest.mark.gpu
def test_results_do_not_depend_on_the_tuning(atmo, oracle, torch_cuda):
    from test_gpu_parity import random_atmosphere
    rng = np.random.default_rng(17)
    atm = random_atmosphere(oracle, rng)
    kinds = (atmo.LUT_TRANSMITTANCE, atmo.LUT_SCATTERING, atmo.LUT_IRRADIANCE)

    def luts(shape):
        b = atmo.Batch([atm], [shape], 4)
        b.run()
        atmo.synchronize_stream()
        return [b.read(0, k) for k in kinds]

    for shape, tunings in ((SMALL, [(1, 1, 1, 1), (4, 8, 2, 3), (2, 6, 4, 4)]),
                           (MEDIUM, [(1, 1, 1, 1), (2, 2, 1, 4), (1, 4, 2, 2)])):
        atmo.set_tuning(shape, None)
        ref = luts(shape)
        for t in tunings:
            atmo.set_tuning(shape, atmo.Tuning(*t))
            for a, b in zip(luts(shape), ref):
                np.testing.assert_array_equal(a, b)
        atmo.set_tuning(shape, None)


@pytest.mark.gpu
def test_autotune_registers_a_launchable_choice(atmo, oracle, torch_cuda):
    t = atmo.autotune(oracle.earth_atmosphere(), MEDIUM, instances=2)
    assert t.multiple_rows >= 1 and t.single_rows >= 1
    assert t.multiple_ms > 0 and t.single_ms > 0
    got = atmo.get_tuning(MEDIUM)
    assert (got.multiple_rows, got.multiple_group) == (t.multiple_rows, t.multiple_group)
    atmo.set_tuning(MEDIUM, None)
