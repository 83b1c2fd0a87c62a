"""Freezes the operation counts of the reference's precomputation algorithm, as
the oracle restates it, for the four precomputation configurations:
tests/golden/flops_config{0..3}.json.

The counts come from the oracle's counting build (oracle/atmo_oracle_count.cc:
atmo_oracle.cc compiled with a scalar type that tallies every operation).  A
FLOP is an add or a mul of the shader arithmetic; divisions, square roots,
exp / pow / sin / cos and compares are counted apart, and texture filtering
(GL LINEAR, done by the texture unit in the reference's shaders) is kept
apart from the shader arithmetic.

Per pass, the operations of a texel depend only on its geometry (no branch
reads a LUT value), so a pass is counted on a systematic sample of its texels
(every stride-th, stride prime) evaluated on LUTs of ones, scaled to all
texels; the luminance products and blending that follow each texel evaluation
(a constant per texel) are taken from an exact run at the small shape.
`--exact` also runs the whole configuration-0 precomputation through the
counting build (~45 min on 8 cores) and records its exact totals beside the
sampled ones.

    python tests/golden/make_flops.py [--exact]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

DEFAULT = (256, 64, 32, 128, 32, 8, 64, 16)      # atmosphere/constants.h:47-61
HALF = (128, 32, 16, 64, 16, 4, 32, 8)
DOUBLE_R = (256, 64, 64, 128, 32, 8, 64, 16)
HIRES = (512, 128, 64, 256, 64, 16, 128, 32)

# Quadrature units per texel (functions.glsl: SAMPLE_COUNT of each integral).
UNITS = {
    "transmittance": (3 * 501, "optical-depth sample (3 profiles x 501 points)"),
    "direct_irradiance": (1, "texel"),
    "single_scattering": (51, "ray sample"),
    "scattering_density": (16 * 32, "direction sample"),
    "indirect_irradiance": (16 * 64, "hemisphere sample"),
    "multiple_scattering": (51, "ray sample"),
}
KIND = {"transmittance": 0, "direct_irradiance": 1, "single_scattering": 2,
        "scattering_density": 3, "indirect_irradiance": 4, "multiple_scattering": 5}
STRIDES = {"transmittance": 7, "direct_irradiance": 1, "single_scattering": 61,
           "scattering_density": 127, "indirect_irradiance": 1, "multiple_scattering": 61}
# Per planet of configuration 3 (the sum over 256 planets averages further).
PLANET_STRIDES = {"transmittance": 97, "direct_irradiance": 1, "single_scattering": 1021,
                  "scattering_density": 2039, "indirect_irradiance": 7,
                  "multiple_scattering": 1021}


def flops(c):
    return c["add"] + c["mul"]


def add_into(acc, c, scale=1.0):
    for cat in ("shader", "filter"):
        for op, v in c[cat].items():
            acc[cat][op] = acc[cat].get(op, 0.0) + v * scale


def empty():
    return {"shader": {}, "filter": {}}


def blend_extras(threads):
    """Operations per texel that follow the texel evaluations in a pass (the
    luminance products and blending of atmosphere/model.cc:1082-1083 as the
    oracle's Precompute does them): an exact small-shape run minus the sum of
    its texel evaluations.  Keyed by (pass, blend)."""
    atm = O.earth_atmosphere()
    shp = O.shape(*O.SMALL_SHAPE)
    n = {"single_scattering": shp.s_size, "indirect_irradiance": shp.i_size,
         "multiple_scattering": shp.s_size}
    orders = 3
    evals = {
        "single_scattering": [O.count_texels(atm, shp, 2, 0, np.arange(shp.s_size), threads)],
        "indirect_irradiance": [O.count_texels(atm, shp, 4, o - 1, np.arange(shp.i_size),
                                               threads) for o in range(2, orders + 1)],
        "multiple_scattering": [O.count_texels(atm, shp, 5, 0, np.arange(shp.s_size), threads)
                                for _ in range(2, orders + 1)],
    }
    out = {}
    for blend in (False, True):
        base = O.precompute(atm, shp, orders, combined=True)
        full = O.count_ops(atm, shp, orders, blend=blend, combined=True, threads=threads,
                           out=base if blend else None)
        for name, parts in evals.items():
            per = empty()
            for cat in ("shader", "filter"):
                for op in O.COUNT_OPS:
                    tot = full[name][cat][op] - sum(p[cat][op] for p in parts)
                    per[cat][op] = tot / (n[name] * len(parts))
            out[(name, blend)] = per
    return out


def pass_sample(atm, shp, name, order, threads, strides):
    """Per-texel average operations of one pass launch, from a strided sample."""
    n = {"transmittance": shp.t_size, "direct_irradiance": shp.i_size,
         "indirect_irradiance": shp.i_size}.get(name, shp.s_size)
    stride = strides[name]
    idx = np.arange(stride // 2 if stride > 1 else 0, n, stride)
    c = O.count_texels(atm, shp, KIND[name], order, idx, threads)
    per = empty()
    add_into(per, c, 1.0 / len(idx))
    return per, n, len(idx)


def config_counts(atm, shape, orders, threads, extras, groups=1, extra_transmittance=0,
                  cache=None, strides=STRIDES):
    """Operations of one configuration: per pass launch (texels x the sampled
    per-texel average, plus the per-texel blending), and the totals."""
    shp = O.shape(*shape)
    cache = {} if cache is None else cache
    launches = []

    def launch(name, order, count, blend):
        key = (tuple(shape), name, order, id(atm))
        if key not in cache:
            cache[key] = pass_sample(atm, shp, name, order, threads, strides)
        per, n, sampled = cache[key]
        ops = empty()
        add_into(ops, per, n)
        if (name, blend) in extras:
            add_into(ops, extras[(name, blend)], n)
        units, unit = UNITS[name]
        launches.append({"pass": name, "order": order, "launches": count, "texels": n,
                         "sampled_texels": sampled, "units_per_texel": units, "unit": unit,
                         "flops": flops(ops["shader"]),
                         "flops_per_unit": flops(ops["shader"]) / (n * units),
                         "filter_flops": flops(ops["filter"]),
                         "shader": ops["shader"], "filter": ops["filter"]})

    for g in range(groups):
        blend = g > 0
        launch("transmittance", 0, 1, blend)
        launch("direct_irradiance", 0, 1, blend)
        launch("single_scattering", 0, 1, blend)
        for order in range(2, orders + 1):
            launch("scattering_density", min(order, 3), 1, blend)
            launch("indirect_irradiance", min(order - 1, 2), 1, blend)
            launch("multiple_scattering", 0, 1, blend)
    for _ in range(extra_transmittance):
        launch("transmittance", 0, 1, False)
    # Merge identical launches (same pass, order and blending) into counts.
    merged = {}
    for l in launches:
        key = (l["pass"], l["order"], json.dumps(l["shader"], sort_keys=True))
        if key in merged:
            merged[key]["launches"] += 1
        else:
            merged[key] = l
    total = empty()
    for l in launches:
        add_into(total, {"shader": l["shader"], "filter": l["filter"]})
    return {"launches": list(merged.values()),
            "total": {"flops": flops(total["shader"]), "filter_flops": flops(total["filter"]),
                      "shader": total["shader"], "filter": total["filter"]}}


def rounded(x):
    if isinstance(x, dict):
        return {k: rounded(v) for k, v in x.items()}
    if isinstance(x, list):
        return [rounded(v) for v in x]
    if isinstance(x, float):
        return float("%.6g" % x)
    return x


def write(n, body):
    path = os.path.join(HERE, "flops_config%d.json" % n)
    with open(path, "w") as f:
        json.dump(rounded(body), f, indent=1, sort_keys=False)
        f.write("\n")
    print("wrote", path, "total %.4g FLOP" % body["counts"]["total"]["flops"])


COMMON = {
    "generator": "tests/golden/make_flops.py (oracle/atmo_oracle_count.cc)",
    "flop": "add or mul of the shader arithmetic (a GPU FMA = its mul + its add); "
            "div, sqrt, exp, pow, sin, cos, floor, fmod and cmp counted apart; texture "
            "filtering (GL LINEAR) apart from the shader arithmetic",
    "method": "per pass: every stride-th texel (stride %s) on LUTs of ones, scaled to all "
              "texels; blending per texel from an exact small-shape run" % STRIDES,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--exact", action="store_true",
                    help="also count the whole configuration-0 precomputation exactly")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--configs", default="0,1,2,3", help="configurations to write")
    args = ap.parse_args()
    which = {int(x) for x in args.configs.split(",")}
    th = args.threads
    t0 = time.time()
    extras = blend_extras(th)
    cache = {}

    # Config 0: the reference's Earth, default shape, 4 orders, 3 wavelengths.
    earth = O.earth_atmosphere()
    c0 = config_counts(earth, DEFAULT, 4, th, extras, cache=cache)
    body = dict(COMMON, config=0, workload="Earth (demo.cc), default shape, 4 orders, 3 wavelengths, "
                "combined textures", shape=DEFAULT, orders=4, counts=c0)
    if args.exact:
        full = O.count_ops(earth, DEFAULT, 4, combined=True, threads=th)
        exact = empty()
        for name in UNITS:
            add_into(exact, full[name])
        body["exact"] = {"flops": flops(exact["shader"]), "filter_flops": flops(exact["filter"]),
                         "shader": exact["shader"], "filter": exact["filter"],
                         "per_pass_flops": {k: flops(full[k]["shader"]) for k in UNITS}}
    if 0 in which:
        write(0, body)

    # Config 1: 15 wavelengths = 5 groups of the default shape (blending from the
    # second group on) and the transmittance recomputed at the end (model.cc:955-963).
    if 1 in which:
        c1 = config_counts(earth, DEFAULT, 4, th, extras, groups=5, extra_transmittance=1,
                           cache=cache)
        write(1, dict(COMMON, config=1, workload="Earth, 15 wavelengths (5 groups of 3), "
                      "default shape, 4 orders", shape=DEFAULT, orders=4, groups=5, counts=c1))

    # Config 2: high-resolution shape, 8 orders, g = 0.76, albedo 0.3.
    if 2 in which:
        hires = O.earth_atmosphere(mie_g=0.76, ground_albedo=0.3)
        c2 = config_counts(hires, HIRES, 8, th, extras, cache=cache)
        write(2, dict(COMMON, config=2, workload="Earth (g 0.76, albedo 0.3), high-resolution "
                      "shape, 8 orders", shape=HIRES, orders=8, counts=c2))

    # Config 3: the 256 seeded planets of the mixed batch (seed 3, as the
    # benchmark draws them), each counted on its own atmosphere and shape.
    if 3 not in which:
        print("done in %.0f s" % (time.time() - t0))
        return
    from precomputed_atmospheric_scattering_gb300 import workloads as W
    import ctypes as C
    rng = np.random.default_rng(3)
    total = empty()
    per_shape = {}
    for q in range(256):
        a, shape, orders = W.random_rebuild(rng)
        atm = O.Atmosphere()
        C.memmove(C.byref(atm), C.byref(a), C.sizeof(O.Atmosphere))
        c = config_counts(atm, shape, orders, th, extras, cache={}, strides=PLANET_STRIDES)
        add_into(total, c["total"])
        key = "%s x %d orders" % ({HALF: "half", DEFAULT: "default",
                                   DOUBLE_R: "double-R"}[tuple(shape)], orders)
        per_shape[key] = per_shape.get(key, 0) + 1
    c3 = {"total": {"flops": flops(total["shader"]), "filter_flops": flops(total["filter"]),
                    "shader": total["shader"], "filter": total["filter"]},
          "instances": per_shape}
    write(3, dict(COMMON, config=3, workload="256 seeded planets (seed 3) of {half, default, "
                  "double-R} shapes, 2-6 orders", counts=c3,
                  method=COMMON["method"].replace(str(STRIDES), str(PLANET_STRIDES))))
    print("done in %.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main()
