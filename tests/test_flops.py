"""The reference algorithm's operation counts (tests/golden/flops_config*.json,
frozen by tests/golden/make_flops.py from the oracle's counting build,
oracle/atmo_oracle_count.cc) and the machinery behind them: the counting build
computes the oracle's LUTs bit for bit; a pass's counts are those of its texel
evaluations, whatever the LUT values (no branch reads them), so sampled texels
on LUTs of ones stand for the real pass; and a fresh sample at the default
shape reproduces the frozen per-unit figures that bench.py's roofline uses."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEFAULT = (256, 64, 32, 128, 32, 8, 64, 16)


def flops(c):
    return c["add"] + c["mul"]


def frozen(n):
    with open(os.path.join(GOLDEN, "flops_config%d.json" % n)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def small_counts(oracle):
    O = oracle
    atm = O.earth_atmosphere(mie_g=0.7, ground_albedo=0.3)
    shp = O.shape(*O.SMALL_SHAPE)
    out = O.Luts(shp)
    counts = O.count_ops(atm, shp, 3, combined=False, out=out)
    return atm, shp, out, counts


def test_counting_build_computes_the_oracle_luts(oracle, small_counts):
    atm, shp, out, _ = small_counts
    ref = oracle.precompute(atm, shp, 3, combined=False)
    for name in ("transmittance", "scattering", "single_mie", "irradiance"):
        np.testing.assert_array_equal(getattr(out, name), getattr(ref, name), err_msg=name)


def test_pass_counts_are_the_texel_evaluations(oracle, small_counts):
    """The full run (real LUT values) against its texels evaluated on LUTs of
    ones: transmittance, direct irradiance and density have no per-texel work
    besides the evaluation, so they agree exactly, op by op."""
    O = oracle
    atm, shp, _, full = small_counts
    nT, nI, nS = shp.t_size, shp.i_size, shp.s_size
    parts = {
        "transmittance": [O.count_texels(atm, shp, 0, 0, np.arange(nT))],
        "direct_irradiance": [O.count_texels(atm, shp, 1, 0, np.arange(nI))],
        "scattering_density": [O.count_texels(atm, shp, 3, o, np.arange(nS)) for o in (2, 3)],
    }
    for name, ps in parts.items():
        assert full[name]["texels"] == sum(p["texels"] for p in ps)
        for cat in ("shader", "filter"):
            for op in O.COUNT_OPS:
                assert full[name][cat][op] == sum(p[cat][op] for p in ps), (name, cat, op)
    # Order 2 evaluates two single-scattering tables with their phase
    # functions, higher orders one table: more work per sample at order 2.
    d2, d3 = parts["scattering_density"]
    assert flops(d2["shader"]) > flops(d3["shader"]) > 0


def test_frozen_per_unit_figures_reproduce(oracle):
    """A fresh, sparser sample at the default shape against the frozen
    configuration-0 figures (those in bench.py's roofline): within 1%."""
    O = oracle
    atm = O.earth_atmosphere()
    shp = O.shape(*DEFAULT)
    launches = {(l["pass"], l["order"]): l for l in frozen(0)["counts"]["launches"]}
    checks = [("scattering_density", 3, 2, 4099, 512), ("scattering_density", 3, 3, 4099, 512),
              ("single_scattering", 2, 0, 4099, 51), ("multiple_scattering", 5, 0, 4099, 51),
              ("transmittance", 0, 0, 97, 1503)]
    for name, kind, order, stride, units in checks:
        n = shp.t_size if kind == 0 else shp.s_size
        idx = np.arange(stride // 3, n, stride)
        c = O.count_texels(atm, shp, kind, order, idx)
        got = flops(c["shader"]) / (len(idx) * units)
        # (The frozen figures of single and multiple scattering also hold the
        # luminance product and blending after each texel: ~0.5 FLOP a sample.)
        want = launches[(name, order)]["flops_per_unit"]
        assert abs(got - want) <= 0.01 * want, (name, got, want)


def test_frozen_totals_are_the_sum_of_their_launches():
    for n in (0, 1, 2):
        c = frozen(n)["counts"]
        total = sum(l["flops"] * l["launches"] for l in c["launches"])
        assert abs(total - c["total"]["flops"]) <= 1e-5 * total, n
        for l in c["launches"]:
            assert abs(l["flops_per_unit"] * l["texels"] * l["units_per_texel"] - l["flops"]) \
                <= 1e-5 * l["flops"]
    # Configuration 1 is five groups of configuration 0's passes plus one
    # transmittance pass; configuration 3 sums 256 planets of three shapes.
    c0, c1 = frozen(0)["counts"]["total"]["flops"], frozen(1)["counts"]["total"]["flops"]
    assert 4.9 * c0 < c1 < 5.1 * c0
    c3 = frozen(3)["counts"]
    assert sum(c3["instances"].values()) == 256
