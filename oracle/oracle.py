"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/libatmo_oracle.so (the double-precision restatement of the
reference's precomputation, oracle/atmo_oracle.cc) and, when it was built in a
container holding the reference sources, oracle/_ref/libatmo_ref.so (the
reference's own atmosphere/functions.glsl compiled as C++ over
oracle/ref/ref_shim.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The product library never calls into it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libatmo_oracle.so")
ORACLE_GPU_SO = os.path.join(HERE, "_build", "libatmo_oracle_gpu.so")
ORACLE_COUNT_SO = os.path.join(HERE, "_build", "libatmo_oracle_count.so")
REF_SO = os.path.join(HERE, "_ref", "libatmo_ref.so")


class Layer(C.Structure):
    """atmosphere/definitions.glsl:185-191 (DensityProfileLayer)."""
    _fields_ = [("width", C.c_double), ("exp_term", C.c_double), ("exp_scale", C.c_double),
                ("linear_term", C.c_double), ("constant_term", C.c_double)]


class Profile(C.Structure):
    """atmosphere/definitions.glsl:197-199 (DensityProfile, two layers)."""
    _fields_ = [("layers", Layer * 2)]


D3 = C.c_double * 3


class Atmosphere(C.Structure):
    """atmosphere/definitions.glsl:205-255 (AtmosphereParameters at 3 wavelengths)."""
    _fields_ = [
        ("solar_irradiance", D3), ("sun_angular_radius", C.c_double),
        ("bottom_radius", C.c_double), ("top_radius", C.c_double),
        ("rayleigh_density", Profile), ("rayleigh_scattering", D3),
        ("mie_density", Profile), ("mie_scattering", D3), ("mie_extinction", D3),
        ("mie_phase_function_g", C.c_double),
        ("absorption_density", Profile), ("absorption_extinction", D3),
        ("ground_albedo", D3), ("mu_s_min", C.c_double),
    ]


class Shape(C.Structure):
    """atmosphere/constants.h:47-61 as run-time values."""
    _fields_ = [("transmittance_width", C.c_int), ("transmittance_height", C.c_int),
                ("scattering_r", C.c_int), ("scattering_mu", C.c_int),
                ("scattering_mu_s", C.c_int), ("scattering_nu", C.c_int),
                ("irradiance_width", C.c_int), ("irradiance_height", C.c_int)]

    @property
    def t_size(self):
        return self.transmittance_width * self.transmittance_height

    @property
    def i_size(self):
        return self.irradiance_width * self.irradiance_height

    @property
    def s_width(self):
        return self.scattering_nu * self.scattering_mu_s

    @property
    def s_size(self):
        return self.s_width * self.scattering_mu * self.scattering_r

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)


def shape(tw, th, r, mu, mu_s, nu, iw, ih) -> Shape:
    return Shape(tw, th, r, mu, mu_s, nu, iw, ih)


DEFAULT_SHAPE = (256, 64, 32, 128, 32, 8, 64, 16)   # atmosphere/constants.h:47-61
MEDIUM_SHAPE = (128, 32, 8, 32, 16, 8, 32, 8)
SMALL_SHAPE = (64, 16, 4, 16, 8, 4, 16, 4)
HIRES_SHAPE = (512, 128, 64, 256, 64, 16, 128, 32)  # high-resolution Earth LUTs


def layer(width=0.0, exp_term=0.0, exp_scale=0.0, linear_term=0.0, constant_term=0.0):
    return Layer(width, exp_term, exp_scale, linear_term, constant_term)


def profile(*layers) -> Profile:
    """Up to two layers, bottom first; missing bottom layers are zero
    (atmosphere/model.cc:676-690 pads at the front)."""
    ls = list(layers)
    while len(ls) < 2:
        ls.insert(0, Layer())
    p = Profile()
    p.layers[0], p.layers[1] = ls[0], ls[1]
    return p


def _d3(v):
    if isinstance(v, (int, float)):
        v = (v, v, v)
    return D3(*[float(x) for x in v])


def atmosphere(**kw) -> Atmosphere:
    a = Atmosphere()
    for k, v in kw.items():
        if isinstance(getattr(a, k), C.Array):
            setattr(a, k, _d3(v))
        else:
            setattr(a, k, v)
    return a


def earth_atmosphere(mie_g=0.8, ground_albedo=0.1, max_sun_zenith_deg=102.0, ozone=True):
    """The Earth atmosphere of atmosphere/demo/demo.cc:188-284 at 680/550/440 nm,
    constant solar spectrum 1.5, in km (length_unit_in_meters = 1000)."""
    lambdas = (680.0, 550.0, 440.0)
    rayleigh = [1.24062e-6 * (l * 1e-3) ** -4 * 1000.0 for l in lambdas]
    mie_ext = 5.328e-3 / 1200.0 * 1000.0
    ozone_xs = {680.0: 1.209e-25, 550.0: 3.5e-25, 440.0: 1.582e-26}
    max_ozone = 300.0 * 2.687e20 / 15000.0
    absorption = [max_ozone * ozone_xs[l] * 1000.0 if ozone else 0.0 for l in lambdas]
    return atmosphere(
        solar_irradiance=1.5, sun_angular_radius=0.00935 / 2.0,
        bottom_radius=6360.0, top_radius=6420.0,
        rayleigh_density=profile(layer(0.0, 1.0, -1.0 / 8.0, 0.0, 0.0)),
        rayleigh_scattering=rayleigh,
        mie_density=profile(layer(0.0, 1.0, -1.0 / 1.2, 0.0, 0.0)),
        mie_scattering=mie_ext * 0.9, mie_extinction=mie_ext,
        mie_phase_function_g=mie_g,
        absorption_density=profile(layer(25.0, 0.0, 0.0, 1.0 / 15.0, -2.0 / 3.0),
                                   layer(0.0, 0.0, 0.0, -1.0 / 15.0, 8.0 / 3.0)),
        absorption_extinction=absorption, ground_albedo=ground_albedo,
        mu_s_min=math.cos(max_sun_zenith_deg / 180.0 * math.pi))


def toy_atmosphere():
    """The fixture planet of atmosphere/reference/functions_test.cc:49-61 and
    :296-313 (spectral values only at the first wavelength, in metres)."""
    km = 1000.0
    return atmosphere(
        solar_irradiance=(123.0, 0.0, 0.0), sun_angular_radius=0.0,
        bottom_radius=1000.0 * km, top_radius=1500.0 * km,
        rayleigh_density=profile(Layer(), layer(0.0, 1.0, -1.0 / (60.0 * km), 0.0, 0.0)),
        rayleigh_scattering=(0.001 / km, 0.0, 0.0),
        mie_density=profile(Layer(), layer(0.0, 1.0, -1.0 / (30.0 * km), 0.0, 0.0)),
        mie_scattering=(0.0015 / km, 0.0, 0.0), mie_extinction=(0.002 / km, 0.0, 0.0),
        mie_phase_function_g=0.0, absorption_density=profile(),
        absorption_extinction=(0.0, 0.0, 0.0), ground_albedo=(0.1, 0.0, 0.0), mu_s_min=-1.0)


def reference_dir():
    """The reference's source checkout, or None: ATMO_REFERENCE_DIR when set
    (it must then hold atmosphere/functions.glsl), else a checkout named
    `reference` beside this repository's directory when there is one.  The
    GPU host has neither, and the oracle then runs without the reference
    build."""
    env = os.environ.get("ATMO_REFERENCE_DIR")
    if env:
        if not os.path.isfile(os.path.join(env, "atmosphere", "functions.glsl")):
            raise RuntimeError("ATMO_REFERENCE_DIR=%s holds no atmosphere/functions.glsl" % env)
        return env
    sibling = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    if os.path.isfile(os.path.join(sibling, "atmosphere", "functions.glsl")):
        return sibling
    return None


def build(quiet=True):
    """Compiles the oracle restatement (and, when the reference sources are
    present, the reference's own functions.glsl) for this machine."""
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    src = os.path.join(HERE, "atmo_oracle.cc")
    if (not os.path.exists(ORACLE_SO)
            or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src)):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC",
                               "-shared", "-pthread", src, "-o", ORACLE_SO])
    gpu_src = os.path.join(HERE, "atmo_oracle_gpu.cu")
    stale = lambda so: (not os.path.exists(so) or  # noqa: E731
                        os.path.getmtime(so) < max(os.path.getmtime(src),
                                                   os.path.getmtime(gpu_src)))
    if stale(ORACLE_GPU_SO):
        # The FP64 GPU oracle: the same evaluators as device code, no FMA
        # contraction (as the CPU build).
        subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                               "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                               gpu_src, "-o", ORACLE_GPU_SO])
    ref_src = reference_dir()
    if ref_src is not None:
        subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"),
                               "REFERENCE=" + ref_src],
                              stdout=subprocess.DEVNULL if quiet else None)


_lib = None
_ref = None
P = C.POINTER
dp = P(C.c_double)


def _arr(x):
    return x.ctypes.data_as(dp) if x is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        A, S = P(Atmosphere), P(Shape)
        d, i = C.c_double, C.c_int
        sig = {
            "oracle_distance_to_top": (d, [A, d, d]),
            "oracle_distance_to_bottom": (d, [A, d, d]),
            "oracle_ray_intersects_ground": (i, [A, d, d]),
            "oracle_distance_to_nearest": (d, [A, d, d, i]),
            "oracle_profile_density": (d, [P(Profile), d]),
            "oracle_optical_length": (d, [A, P(Profile), d, d]),
            "oracle_transmittance_to_top": (None, [A, d, d, dp]),
            "oracle_tex_coord_from_unit_range": (d, [d, i]),
            "oracle_unit_range_from_tex_coord": (d, [d, i]),
            "oracle_transmittance_uv_from_rmu": (None, [A, S, d, d, dp]),
            "oracle_rmu_from_transmittance_uv": (None, [A, S, d, d, dp, dp]),
            "oracle_lookup_transmittance_to_top": (None, [A, S, dp, d, d, dp]),
            "oracle_lookup_transmittance": (None, [A, S, dp, d, d, d, i, dp]),
            "oracle_lookup_transmittance_to_sun": (None, [A, S, dp, d, d, dp]),
            "oracle_single_scattering_integrand": (None, [A, S, dp, d, d, d, d, d, i, dp, dp]),
            "oracle_single_scattering": (None, [A, S, dp, d, d, d, d, i, dp, dp]),
            "oracle_rayleigh_phase": (d, [d]),
            "oracle_mie_phase": (d, [d, d]),
            "oracle_scattering_uvwz": (None, [A, S, d, d, d, d, i, dp]),
            "oracle_rmumusnu_from_uvwz": (None, [A, S, dp, dp, P(i)]),
            "oracle_rmumusnu_from_frag_coord": (None, [A, S, dp, dp, P(i)]),
            "oracle_lookup_scattering": (None, [A, S, dp, d, d, d, d, i, dp]),
            "oracle_scattering_taps": (None, [A, S, d, d, d, d, i, P(i), dp]),
            "oracle_scattering_density": (None, [A, S, dp, dp, dp, dp, dp, d, d, d, d, i, dp]),
            "oracle_multiple_scattering": (None, [A, S, dp, dp, d, d, d, d, i, dp]),
            "oracle_direct_irradiance": (None, [A, S, dp, d, d, dp]),
            "oracle_indirect_irradiance": (None, [A, S, dp, dp, dp, d, d, i, dp]),
            "oracle_irradiance_uv_from_rmus": (None, [A, S, d, d, dp]),
            "oracle_rmus_from_irradiance_uv": (None, [A, S, d, d, dp, dp]),
            "oracle_lookup_irradiance": (None, [A, S, dp, d, d, dp]),
            "oracle_eval_texels": (None, [i, A, S, dp, dp, dp, dp, dp, dp, i, i,
                                          P(C.c_longlong), dp, dp, i]),
            "oracle_precompute": (i, [A, S, C.c_uint, dp, i, i, i, dp, dp, dp, dp]),
            "oracle_time_precompute_sample": (i, [A, S, C.c_uint, i, i, dp]),
            "oracle_time_precompute_partitioned": (i, [A, S, C.c_uint, i, i, i, dp]),
            "oracle_interpolate": (d, [dp, dp, i, d]),
            "oracle_cie_table_value": (d, [d, i]),
            "oracle_radiance_to_luminance_factors": (None, [dp, dp, i, d, dp]),
            "oracle_convert_spectrum_to_linear_srgb": (None, [dp, dp, i, dp]),
            "oracle_sky_radiance": (None, [A, S, dp, dp, dp, i, dp, dp, d, dp, dp, dp]),
            "oracle_sky_radiance_to_point": (None, [A, S, dp, dp, dp, i, dp, dp, d, dp, dp, dp]),
            "oracle_sun_and_sky_irradiance": (None, [A, S, dp, dp, dp, dp, dp, dp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


_gpu = None


def gpu_lib():
    """The FP64 GPU oracle (atmo_oracle_gpu.cu): the CPU oracle's evaluators
    as device code, for LUT shapes too large for the CPU."""
    global _gpu
    if _gpu is None:
        if not os.path.exists(ORACLE_GPU_SO):
            build()
        L = C.CDLL(ORACLE_GPU_SO)
        L.oracle_gpu_precompute.restype = C.c_int
        L.oracle_gpu_precompute.argtypes = [P(Atmosphere), P(Shape), C.c_uint, dp, C.c_int,
                                            C.c_int, dp, dp, dp, dp]
        _gpu = L
    return _gpu


def gpu_precompute(atm: Atmosphere, shp, orders=4, lum=None, blend=False, combined=True,
                   out: Luts | None = None) -> Luts:
    """precompute() on the GPU in FP64 (needs a CUDA device)."""
    if not isinstance(shp, Shape):
        shp = shape(*shp)
    out = out or Luts(shp)
    lum = np.ascontiguousarray(IDENTITY if lum is None else np.asarray(lum, np.float64).reshape(9))
    rc = gpu_lib().oracle_gpu_precompute(C.byref(atm), C.byref(shp), orders, _arr(lum),
                                         int(blend), int(combined), _arr(out.transmittance),
                                         _arr(out.scattering),
                                         _arr(None if combined else out.single_mie),
                                         _arr(out.irradiance))
    if rc != 0:
        raise RuntimeError("GPU oracle precompute failed")
    return out


_count = None

# Operation kinds and buckets of the FLOP-counting build (atmo_oracle_count.cc).
COUNT_OPS = ("add", "mul", "div", "sqrt", "exp", "pow", "sin", "cos", "floor", "fmod", "cmp")
COUNT_PASSES = ("transmittance", "direct_irradiance", "single_scattering",
                "scattering_density", "indirect_irradiance", "multiple_scattering", "host")


def count_lib():
    """The oracle compiled with a counting scalar type (atmo_oracle_count.cc);
    built on first use."""
    global _count
    if _count is None:
        src = os.path.join(HERE, "atmo_oracle_count.cc")
        deps = [src, os.path.join(HERE, "atmo_oracle.cc"), os.path.join(HERE, "atmo_oracle.h")]
        if (not os.path.exists(ORACLE_COUNT_SO) or
                os.path.getmtime(ORACLE_COUNT_SO) < max(map(os.path.getmtime, deps))):
            os.makedirs(os.path.dirname(ORACLE_COUNT_SO), exist_ok=True)
            subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC",
                                   "-shared", "-pthread", src, "-o", ORACLE_COUNT_SO])
        L = C.CDLL(ORACLE_COUNT_SO)
        L.oracle_precompute.restype = C.c_int
        L.oracle_precompute.argtypes = [P(Atmosphere), P(Shape), C.c_uint, dp, C.c_int, C.c_int,
                                        C.c_int, dp, dp, dp, dp]
        L.oracle_time_precompute_sample.restype = C.c_int
        L.oracle_time_precompute_sample.argtypes = [P(Atmosphere), P(Shape), C.c_uint, C.c_int,
                                                    C.c_int, dp]
        L.oracle_count_reset.argtypes = []
        L.oracle_count_dims.argtypes = [P(C.c_int)]
        L.oracle_count_read.argtypes = [P(C.c_ulonglong), P(C.c_ulonglong)]
        _count = L
    return _count


def _read_counts(L):
    dims = (C.c_int * 3)()
    L.oracle_count_dims(dims)
    nb, nf, no = dims
    assert (nb, nf, no) == (len(COUNT_PASSES), 2, len(COUNT_OPS))
    counts = np.zeros(nb * nf * no, np.uint64)
    calls = np.zeros(nb, np.uint64)
    L.oracle_count_read(counts.ctypes.data_as(P(C.c_ulonglong)),
                        calls.ctypes.data_as(P(C.c_ulonglong)))
    counts = counts.reshape(nb, nf, no)
    out = {}
    for b, name in enumerate(COUNT_PASSES):
        out[name] = {"texels": int(calls[b]),
                     "shader": {op: int(counts[b, 0, o]) for o, op in enumerate(COUNT_OPS)},
                     "filter": {op: int(counts[b, 1, o]) for o, op in enumerate(COUNT_OPS)}}
    return out


def count_ops(atm: Atmosphere, shp, orders=4, lum=None, blend=False, combined=True,
              threads=0, stride=1, out: Luts | None = None):
    """Runs precompute() through the counting build and returns, per pass, the
    texel evaluations and the operations by kind, shader arithmetic and texture
    filtering apart.  stride > 1 evaluates every stride-th texel of the
    density and multiple-scattering passes only (a sample, identity luminance,
    separate single Mie; their per-texel averages stand for the full pass).
    With stride 1 the LUTs (in `out`) equal precompute()'s; with combined
    textures no single-Mie table is written, as in the reference."""
    if not isinstance(shp, Shape):
        shp = shape(*shp)
    L = count_lib()
    L.oracle_count_reset()
    if stride > 1:
        seconds = np.zeros(6)
        rc = L.oracle_time_precompute_sample(C.byref(atm), C.byref(shp), orders, stride,
                                             threads, _arr(seconds))
    else:
        out = out or Luts(shp)
        lum = np.ascontiguousarray(IDENTITY if lum is None
                                   else np.asarray(lum, np.float64).reshape(9))
        rc = L.oracle_precompute(C.byref(atm), C.byref(shp), orders, _arr(lum), int(blend),
                                 int(combined), threads, _arr(out.transmittance),
                                 _arr(out.scattering),
                                 _arr(None if combined else out.single_mie),
                                 _arr(out.irradiance))
    if rc != 0:
        raise RuntimeError("counting oracle precompute failed: %d" % rc)
    return _read_counts(L)


def count_texels(atm: Atmosphere, shp, kind, order, idx, threads=0):
    """The operations of evaluating texels idx of pass `kind` (0 transmittance,
    1 direct irradiance, 2 single scattering, 3 scattering density, 4 indirect
    irradiance, 5 multiple scattering; `order` as the pass takes it) through
    the counting build, as count_ops() reports one pass.  The input LUTs hold
    ones: no branch of the evaluators depends on LUT values, only on the
    geometry, so the counts are those of the real pass at these texels."""
    if not isinstance(shp, Shape):
        shp = shape(*shp)
    L = count_lib()
    if not hasattr(L, "_eval_sig"):
        L.oracle_eval_texels.restype = None
        L.oracle_eval_texels.argtypes = [C.c_int, P(Atmosphere), P(Shape), dp, dp, dp, dp, dp,
                                         dp, C.c_int, C.c_int, P(C.c_longlong), dp, dp, C.c_int]
        L._eval_sig = True
    T = np.ones(shp.t_size * 4)
    S = np.ones(shp.s_size * 4)
    I = np.ones(shp.i_size * 4)
    idx = np.ascontiguousarray(idx, np.int64)
    out = np.zeros(4 * len(idx))
    out2 = np.zeros(4 * len(idx))
    L.oracle_count_reset()
    L.oracle_eval_texels(kind, C.byref(atm), C.byref(shp), _arr(T), _arr(S), _arr(S), _arr(S),
                         _arr(I), _arr(S), order, len(idx),
                         idx.ctypes.data_as(P(C.c_longlong)), _arr(out), _arr(out2), threads)
    return _read_counts(L)[COUNT_PASSES[kind]]


def ref_lib():
    """The reference's own functions.glsl compiled as C++, or None when it was
    not built on this machine (the reference sources are absent)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        try:
            L = C.CDLL(REF_SO)
        except OSError:
            return None
        A, S = P(Atmosphere), P(Shape)
        d, i = C.c_double, C.c_int
        L.ref_has_shape.restype = i
        L.ref_has_shape.argtypes = [S]
        L.ref_precompute.restype = i
        L.ref_precompute.argtypes = [A, S, C.c_uint, dp, i, i, i, dp, dp, dp, dp]
        L.ref_point_geometry.argtypes = [A, d, d, dp]
        L.ref_transmittance_to_top.argtypes = [A, d, d, dp]
        L.ref_scattering_uvwz.argtypes = [A, S, d, d, d, d, i, dp]
        L.ref_frag_coord_to_rmumusnu.argtypes = [A, S, dp, dp, P(i)]
        L.ref_sky_radiance.argtypes = [A, S, dp, dp, dp, dp, dp, d, dp, dp, dp]
        L.ref_sky_radiance_to_point.argtypes = [A, S, dp, dp, dp, dp, dp, d, dp, dp, dp]
        L.ref_sun_and_sky_irradiance.argtypes = [A, S, dp, dp, dp, dp, dp, dp, dp]
        _ref = L
    return _ref


IDENTITY = np.eye(3).reshape(9)


class Luts:
    """Double RGBA LUTs of one precomputation: transmittance (H_T, W_T, 4),
    scattering and single_mie (R, MU, NU*MU_S, 4), irradiance (H_I, W_I, 4)."""

    def __init__(self, shp: Shape):
        self.shape = shp
        self.transmittance = np.zeros((shp.transmittance_height, shp.transmittance_width, 4))
        self.scattering = np.zeros((shp.scattering_r, shp.scattering_mu, shp.s_width, 4))
        self.single_mie = np.zeros_like(self.scattering)
        self.irradiance = np.zeros((shp.irradiance_height, shp.irradiance_width, 4))


def precompute(atm: Atmosphere, shp, orders=4, lum=None, blend=False, combined=True,
               threads=0, out: Luts | None = None, use_reference=False) -> Luts:
    """Runs the full pass sequence of atmosphere/model.cc:1048-1215 on the CPU."""
    if not isinstance(shp, Shape):
        shp = shape(*shp)
    out = out or Luts(shp)
    lum = np.ascontiguousarray(IDENTITY if lum is None else np.asarray(lum, np.float64).reshape(9))
    args = (C.byref(atm), C.byref(shp), orders, _arr(lum), int(blend), int(combined), threads,
            _arr(out.transmittance), _arr(out.scattering),
            _arr(out.single_mie), _arr(out.irradiance))
    if use_reference:
        L = ref_lib()
        if L is None or not L.ref_has_shape(C.byref(shp)):
            raise RuntimeError("reference build unavailable for this shape")
        rc = L.ref_precompute(*args)
    else:
        rc = lib().oracle_precompute(*args)
    if rc != 0:
        raise RuntimeError("oracle precompute failed: %d" % rc)
    return out


def v3(fn, *args):
    out = np.zeros(3)
    fn(*args, _arr(out))
    return out
