"""GB300-native precomputation of Bruneton's atmospheric-scattering LUTs.

Python mirror of the reference's C++ API (ebruneton/precomputed_atmospheric_
scattering, atmosphere/model.h): ``DensityProfileLayer``, ``Model`` with the
same 19 constructor parameters, ``Model.Init(num_scattering_orders=4)``,
``Model.shader()``, ``Model.SetProgramUniforms`` (unavailable: no graphics
stack), ``Model.ConvertSpectrumToLinearSrgb`` and ``kLambdaR/G/B``.  Every call
goes through the C ABI of include/atmo/atmo.h in libatmo_gb300.so (CUDA for
sm_103a); there is no CPU path: when the library is missing this module raises.

The LUTs stay on the GPU; ``Model.transmittance()`` and friends copy them to
host numpy arrays in the reference's texture layouts (x fastest: transmittance
(H, W, 4), scattering (R, MU, NU*MU_S, 4), irradiance (H, W, 4)).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
# ATMO_LIBRARY=checked loads the checked build (device-side index checks of
# csrc/atmo_check.cuh, built on first use) instead of the ordinary one.
CHECKED = os.environ.get("ATMO_LIBRARY", "") == "checked"
LIB_PATH = os.path.join(_PKG, "libatmo_gb300_checked.so" if CHECKED else "libatmo_gb300.so")

kLambdaR = 680.0
kLambdaG = 550.0
kLambdaB = 440.0

OK, INVALID_ARG, OOM, CUDA_ERROR, TIMEOUT, BUDGET, UNAVAILABLE, NOT_READY, CANCELLED = range(9)
LUT_TRANSMITTANCE, LUT_SCATTERING, LUT_SINGLE_MIE, LUT_IRRADIANCE = range(4)
PATH_FAST, PATH_PLAIN = 0, 1


class AtmoError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("atmo status %d: %s" % (status, message))
        self.status = status


class Unavailable(AtmoError):
    pass


# ---------------------------------------------------------------------------
# C structs of include/atmo/atmo.h
# ---------------------------------------------------------------------------
class _Layer(C.Structure):
    _fields_ = [("width", C.c_double), ("exp_term", C.c_double), ("exp_scale", C.c_double),
                ("linear_term", C.c_double), ("constant_term", C.c_double)]


class _ModelParams(C.Structure):
    _fields_ = [
        ("wavelengths", C.POINTER(C.c_double)), ("num_wavelengths", C.c_uint),
        ("solar_irradiance", C.POINTER(C.c_double)), ("sun_angular_radius", C.c_double),
        ("bottom_radius", C.c_double), ("top_radius", C.c_double),
        ("rayleigh_density", C.POINTER(_Layer)), ("num_rayleigh_layers", C.c_uint),
        ("rayleigh_scattering", C.POINTER(C.c_double)),
        ("mie_density", C.POINTER(_Layer)), ("num_mie_layers", C.c_uint),
        ("mie_scattering", C.POINTER(C.c_double)), ("mie_extinction", C.POINTER(C.c_double)),
        ("mie_phase_function_g", C.c_double),
        ("absorption_density", C.POINTER(_Layer)), ("num_absorption_layers", C.c_uint),
        ("absorption_extinction", C.POINTER(C.c_double)),
        ("ground_albedo", C.POINTER(C.c_double)),
        ("max_sun_zenith_angle", C.c_double), ("length_unit_in_meters", C.c_double),
        ("num_precomputed_wavelengths", C.c_uint),
        ("combine_scattering_textures", C.c_int), ("half_precision", C.c_int),
    ]


class LutShape(C.Structure):
    """atmosphere/constants.h:47-61 as run-time sizes."""
    _fields_ = [("transmittance_width", C.c_int), ("transmittance_height", C.c_int),
                ("scattering_r", C.c_int), ("scattering_mu", C.c_int),
                ("scattering_mu_s", C.c_int), ("scattering_nu", C.c_int),
                ("irradiance_width", C.c_int), ("irradiance_height", C.c_int)]

    @classmethod
    def of(cls, shape):
        if shape is None:
            return None
        if isinstance(shape, cls):
            return shape
        return cls(*[int(v) for v in shape])

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)


DEFAULT_SHAPE = (256, 64, 32, 128, 32, 8, 64, 16)


class _Profile(C.Structure):
    _fields_ = [("layers", _Layer * 2)]


_D3 = C.c_double * 3


class Atmosphere(C.Structure):
    """One wavelength group's AtmosphereParameters (atmosphere/definitions.glsl:
    205-255) at 3 wavelengths, in length units."""
    _fields_ = [
        ("solar_irradiance", _D3), ("sun_angular_radius", C.c_double),
        ("bottom_radius", C.c_double), ("top_radius", C.c_double),
        ("rayleigh_density", _Profile), ("rayleigh_scattering", _D3),
        ("mie_density", _Profile), ("mie_scattering", _D3), ("mie_extinction", _D3),
        ("mie_phase_function_g", C.c_double),
        ("absorption_density", _Profile), ("absorption_extinction", _D3),
        ("ground_albedo", _D3), ("mu_s_min", C.c_double),
    ]

    @classmethod
    def from_buffer_of(cls, other):
        """Copies any ctypes struct with this layout (e.g. the oracle's)."""
        a = cls()
        C.memmove(C.byref(a), C.byref(other), C.sizeof(cls))
        return a


_F3 = C.c_float * 3


class PinholeView(C.Structure):
    """atmo_pinhole_view: a 1920x1080-style pinhole camera for atmo_shade_view."""
    _fields_ = [("camera", _F3), ("right", _F3), ("up", _F3), ("forward", _F3),
                ("fov_y", C.c_float), ("width", C.c_int), ("height", C.c_int),
                ("sun_direction", _F3), ("albedo", _F3)]


class Tuning(C.Structure):
    """atmo_tuning: block shape of the row-restructured kernels for one LUT shape."""
    _fields_ = [("multiple_rows", C.c_int), ("multiple_group", C.c_int),
                ("single_rows", C.c_int), ("single_group", C.c_int),
                ("multiple_ms", C.c_float), ("single_ms", C.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_rebuilds_in_flight", C.c_uint),
                ("shade_streams", C.c_uint), ("combined", C.c_int),
                ("admit_window_us", C.c_uint), ("pool_max_bytes", C.c_size_t),
                ("max_shades_in_flight", C.c_uint)]


class TicketInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("status", C.c_int), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("set_id", C.c_uint64), ("launch_ms", C.c_double),
                ("device_ms", C.c_double), ("rounds", C.c_uint)]


class ServerStats(C.Structure):
    _fields_ = [("used_bytes", C.c_size_t), ("budget_bytes", C.c_size_t),
                ("resident_sets", C.c_uint), ("building", C.c_uint), ("pending", C.c_uint),
                ("evictions", C.c_ulonglong), ("rounds", C.c_ulonglong),
                ("kernels", C.c_ulonglong), ("shades_launched", C.c_ulonglong)]


class PassBuffers(C.Structure):
    """atmo_pass_buffers: device pointers (ints) of one atmo_run_pass."""
    _fields_ = [(n, C.c_void_p) for n in ("transmittance", "delta_rayleigh", "delta_mie",
                                           "delta_irradiance", "delta_density", "scattering",
                                           "irradiance")]


class LutView(C.Structure):
    _fields_ = [("device_ptr", C.c_void_p), ("width", C.c_int), ("height", C.c_int),
                ("depth", C.c_int), ("dtype", C.c_int), ("bytes", C.c_size_t)]


# ---------------------------------------------------------------------------
# Library loading
# ---------------------------------------------------------------------------
_lib = None


def build(verbose=False, force=False, checked=None):
    """Compiles libatmo_gb300.so for sm_103a (nvcc); with checked (default:
    the ATMO_LIBRARY setting), libatmo_gb300_checked.so."""
    from . import nvcc_build as _b
    return _b.build(verbose=verbose, force=force, checked=CHECKED if checked is None else checked)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "%s is not built: run precomputed_atmospheric_scattering_gb300."
                "build() (there is no CPU fallback)" % os.path.basename(LIB_PATH))
        L = C.CDLL(LIB_PATH)
        P, st = C.POINTER, C.c_int
        vp = C.c_void_p
        L.atmo_abi_version.restype = C.c_int
        L.atmo_last_error.restype = C.c_char_p
        sigs = {
            "atmo_synchronize": [vp],
            "atmo_model_create": [P(_ModelParams), P(LutShape), P(vp)],
            "atmo_model_destroy": [vp],
            "atmo_model_init": [vp, C.c_uint, vp],
            "atmo_model_set_path": [vp, C.c_int],
            "atmo_model_set_exact_parameters": [vp, C.c_int],
            "atmo_model_get_lut": [vp, C.c_int, P(LutView)],
            "atmo_model_read_lut": [vp, C.c_int, P(C.c_float), C.c_size_t],
            "atmo_model_atmosphere_at": [vp, P(C.c_double), P(Atmosphere)],
            "atmo_model_shader_source": [vp, C.c_char_p, C.c_size_t, P(C.c_size_t)],
            "atmo_model_luminance_factors": [vp, P(C.c_double), P(C.c_double)],
            "atmo_model_set_program_uniforms": [vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                                C.c_uint],
            "atmo_convert_spectrum_to_linear_srgb": [P(C.c_double), P(C.c_double), C.c_uint,
                                                     P(C.c_double), P(C.c_double),
                                                     P(C.c_double)],
            "atmo_precompute": [P(Atmosphere), P(LutShape), C.c_uint, P(C.c_float), C.c_int,
                                C.c_int, C.c_int, vp, vp, vp, vp, vp],
            "atmo_precompute_noalloc": [P(Atmosphere), P(LutShape), C.c_uint, P(C.c_float),
                                        C.c_int, C.c_int, vp, vp, vp, vp, vp],
            "atmo_run_pass": [P(Atmosphere), P(LutShape), C.c_int, C.c_uint, C.c_int,
                              P(PassBuffers), vp],
            "atmo_batch_create": [P(Atmosphere), P(LutShape), P(C.c_uint), C.c_uint, C.c_int,
                                  P(vp)],
            "atmo_batch_destroy": [vp],
            "atmo_batch_set_atmosphere": [vp, C.c_uint, P(Atmosphere)],
            "atmo_batch_run": [vp, vp],
            "atmo_batch_get_lut": [vp, C.c_uint, C.c_int, P(LutView)],
            "atmo_batch_read_lut": [vp, C.c_uint, C.c_int, P(C.c_float), C.c_size_t],
            "atmo_batch_kernel_count": [vp, P(C.c_uint)],
            "atmo_batch_copy_lut": [vp, C.c_uint, C.c_int, vp, C.c_size_t, vp],
            "atmo_measure_fp32_peak": [P(C.c_double)],
            "atmo_batch_time_passes": [vp, vp, C.c_uint, P(C.c_float), P(C.c_int), P(C.c_int),
                                       P(C.c_uint)],
            "atmo_model_lut_set": [vp, P(vp)],
            "atmo_batch_lut_set": [vp, C.c_uint, P(vp)],
            "atmo_sky_radiance": [vp, vp, vp, vp, vp, C.c_int, C.c_uint, C.c_int, vp, vp, vp],
            "atmo_sky_radiance_to_point": [vp, vp, vp, vp, vp, C.c_int, C.c_uint, C.c_int, vp,
                                           vp, vp],
            "atmo_sun_and_sky_irradiance": [vp, vp, vp, vp, C.c_int, C.c_uint, C.c_int, vp, vp,
                                            vp],
            "atmo_solar_radiance": [vp, C.c_int, P(C.c_double)],
            "atmo_shade_view": [vp, P(PinholeView), vp, C.c_int, vp, vp, vp],
            "atmo_lut_set_read": [vp, C.c_int, P(C.c_float), C.c_size_t],
            "atmo_server_create": [P(ServerConfig), P(vp)],
            "atmo_server_destroy": [vp],
            "atmo_server_submit_rebuild": [vp, P(Atmosphere), P(LutShape), C.c_uint,
                                           P(C.c_uint64)],
            "atmo_server_submit_shade": [vp, C.c_uint64, P(PinholeView), vp, vp, vp,
                                         P(C.c_uint64)],
            "atmo_server_poll": [vp, C.c_uint64, P(TicketInfo)],
            "atmo_server_wait": [vp, C.c_uint64, C.c_uint, P(TicketInfo)],
            "atmo_server_release_ticket": [vp, C.c_uint64],
            "atmo_server_cancel": [vp, C.c_uint64],
            "atmo_server_lut_set": [vp, C.c_uint64, P(vp)],
            "atmo_server_evict": [vp, C.c_uint64],
            "atmo_server_get_stats": [vp, P(ServerStats)],
            "atmo_autotune": [P(Atmosphere), P(LutShape), C.c_uint, P(Tuning)],
            "atmo_device_checks": [C.c_int, P(C.c_int), P(C.c_ulonglong)],
            "atmo_device_checks_selftest": [vp],
            "atmo_set_tuning": [P(LutShape), P(Tuning)],
            "atmo_get_tuning": [P(LutShape), P(Tuning)],
            "atmo_model_save_luts": [vp, C.c_char_p],
            "atmo_model_load_luts": [vp, C.c_char_p],
            "atmo_batch_save_luts": [vp, C.c_uint, C.c_char_p],
        }
        for name, args in sigs.items():
            f = getattr(L, name)
            f.restype = st
            f.argtypes = args
        if L.atmo_abi_version() != 3:
            raise ImportError("libatmo_gb300.so ABI version mismatch")
        _lib = L
    return _lib


def _check(status):
    if status != OK:
        msg = lib().atmo_last_error().decode()
        if status == UNAVAILABLE:
            raise Unavailable(status, msg)
        raise AtmoError(status, msg)


def _dptr(a):
    return np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


# ---------------------------------------------------------------------------
# Reference API
# ---------------------------------------------------------------------------
class DensityProfileLayer:
    """atmosphere/model.h:165-178 (width in m, exp_scale/linear_term in 1/m)."""

    def __init__(self, width=0.0, exp_term=0.0, exp_scale=0.0, linear_term=0.0,
                 constant_term=0.0):
        self.width = width
        self.exp_term = exp_term
        self.exp_scale = exp_scale
        self.linear_term = linear_term
        self.constant_term = constant_term

    def _c(self):
        return _Layer(self.width, self.exp_term, self.exp_scale, self.linear_term,
                      self.constant_term)


def _layers(ls):
    arr = (_Layer * max(1, len(ls)))(*[l._c() for l in ls])
    return arr, len(ls)


class Model:
    """atmosphere/model.h:180-337 over CUDA: the same constructor parameters,
    ``Init``, ``shader`` and LUT layouts; the LUTs are device buffers."""

    kLambdaR = kLambdaR
    kLambdaG = kLambdaG
    kLambdaB = kLambdaB

    def __init__(self, wavelengths, solar_irradiance, sun_angular_radius, bottom_radius,
                 top_radius, rayleigh_density, rayleigh_scattering, mie_density,
                 mie_scattering, mie_extinction, mie_phase_function_g, absorption_density,
                 absorption_extinction, ground_albedo, max_sun_zenith_angle,
                 length_unit_in_meters, num_precomputed_wavelengths,
                 combine_scattering_textures, half_precision, lut_shape=None):
        L = lib()
        n = len(wavelengths)
        self._keep = [np.ascontiguousarray(x, np.float64) for x in (
            wavelengths, solar_irradiance, rayleigh_scattering, mie_scattering,
            mie_extinction, absorption_extinction, ground_albedo)]
        for arr in self._keep:
            if arr.shape != (n,):
                raise ValueError("spectral arrays must have len(wavelengths) entries")
        ray, nr = _layers(rayleigh_density)
        mie, nm = _layers(mie_density)
        ab, na = _layers(absorption_density)
        self._layers = (ray, mie, ab)
        pp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        w, sol, rs, ms, me, ae, ga = self._keep
        p = _ModelParams(pp(w), n, pp(sol), sun_angular_radius, bottom_radius, top_radius,
                         ray, nr, pp(rs), mie, nm, pp(ms), pp(me), mie_phase_function_g,
                         ab, na, pp(ae), pp(ga), max_sun_zenith_angle, length_unit_in_meters,
                         num_precomputed_wavelengths, int(bool(combine_scattering_textures)),
                         int(bool(half_precision)))
        self._shape = LutShape.of(lut_shape) or LutShape(*DEFAULT_SHAPE)
        self.combine_scattering_textures = bool(combine_scattering_textures)
        self.half_precision = bool(half_precision)
        self.num_precomputed_wavelengths = num_precomputed_wavelengths
        h = C.c_void_p()
        _check(L.atmo_model_create(C.byref(p), C.byref(self._shape), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.atmo_model_destroy(h)
            self._h = None

    # --- precomputation -------------------------------------------------------
    def Init(self, num_scattering_orders=4, stream=None, path=None, synchronize=True):
        """atmosphere/model.cc:866-975 on the GPU."""
        if path is not None:
            _check(lib().atmo_model_set_path(self._h, path))
        _check(lib().atmo_model_init(self._h, num_scattering_orders, _stream_ptr(stream)))
        if synchronize:
            synchronize_stream(stream)

    init = Init

    def set_exact_parameters(self, exact=True):
        _check(lib().atmo_model_set_exact_parameters(self._h, int(bool(exact))))

    # --- LUT access -----------------------------------------------------------
    def lut_view(self, kind) -> LutView:
        v = LutView()
        _check(lib().atmo_model_get_lut(self._h, kind, C.byref(v)))
        return v

    def _read(self, kind):
        v = self.lut_view(kind)
        out = np.empty((v.depth, v.height, v.width, 4), np.float32)
        _check(lib().atmo_model_read_lut(self._h, kind,
                                         out.ctypes.data_as(C.POINTER(C.c_float)), out.nbytes))
        return out if v.depth > 1 else out[0]

    def transmittance(self):
        return self._read(LUT_TRANSMITTANCE)

    def scattering(self):
        return self._read(LUT_SCATTERING)

    def single_mie_scattering(self):
        return self._read(LUT_SINGLE_MIE)

    def irradiance(self):
        return self._read(LUT_IRRADIANCE)

    def save_luts(self, directory):
        """transmittance.dat, scattering.dat, irradiance.dat (raw float32 RGBA,
        atmosphere/demo/webgl/precompute.cc:63-106) and atmosphere_shader.txt."""
        _check(lib().atmo_model_save_luts(self._h, os.fsencode(directory)))

    def load_luts(self, directory):
        """Makes the model ready from LUT files instead of Init."""
        _check(lib().atmo_model_load_luts(self._h, os.fsencode(directory)))

    def lut_set(self) -> "LutSet":
        """The render-time query interface of the precomputed LUTs."""
        h = C.c_void_p()
        _check(lib().atmo_model_lut_set(self._h, C.byref(h)))
        return LutSet(h, self, self._shape.as_tuple())

    def atmosphere_at(self, lambdas=(kLambdaR, kLambdaG, kLambdaB)) -> Atmosphere:
        a = Atmosphere()
        _check(lib().atmo_model_atmosphere_at(self._h, _dptr(lambdas), C.byref(a)))
        return a

    def luminance_factors(self):
        sky, sun = (C.c_double * 3)(), (C.c_double * 3)()
        _check(lib().atmo_model_luminance_factors(self._h, sky, sun))
        return tuple(sky), tuple(sun)

    def shader(self) -> str:
        """The GLSL source the reference's shader() compiles (header of
        atmosphere/model.cc:691-744 + API functions); the reference's own
        definitions/functions.glsl text is not bundled and is marked."""
        need = C.c_size_t()
        _check(lib().atmo_model_shader_source(self._h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        _check(lib().atmo_model_shader_source(self._h, buf, need.value, C.byref(need)))
        return buf.value.decode()

    def SetProgramUniforms(self, program, transmittance_texture_unit, scattering_texture_unit,
                           irradiance_texture_unit, single_mie_scattering_texture_unit=0):
        _check(lib().atmo_model_set_program_uniforms(
            self._h, program, transmittance_texture_unit, scattering_texture_unit,
            irradiance_texture_unit, single_mie_scattering_texture_unit))

    @staticmethod
    def ConvertSpectrumToLinearSrgb(wavelengths, spectrum):
        """atmosphere/model.cc:1020-1040; returns (r, g, b)."""
        r, g, b = C.c_double(), C.c_double(), C.c_double()
        _check(lib().atmo_convert_spectrum_to_linear_srgb(
            _dptr(wavelengths), _dptr(spectrum), len(wavelengths), C.byref(r), C.byref(g),
            C.byref(b)))
        return r.value, g.value, b.value


def _tensor_ptr(t, n3=None):
    """Device pointer of a contiguous float32 CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
            and t.is_contiguous()):
        raise ValueError("query arrays must be contiguous float32 CUDA tensors")
    if n3 is not None and t.numel() != 3 * n3:
        raise ValueError("expected %d float triples" % n3)
    return t.data_ptr()


class LutSet:
    """A resident LUT set (a model after Init, or a batch instance after run)
    and the render-time queries of the reference's shader API
    (atmosphere/model.cc:221-281): GetSkyRadiance, GetSkyRadianceToPoint,
    GetSunAndSkyIrradiance, GetSolarRadiance and their luminance forms, as
    CUDA kernels over float32 CUDA tensors of shape (n, 3)."""

    def __init__(self, handle, owner, shape=None):
        self._h = handle
        self._owner = owner   # keeps the model / batch / server alive
        self._owner_shape = tuple(shape) if shape is not None else None

    def _sun(self, sun, n):
        import torch
        if sun.numel() == 3:
            return sun, 0
        _tensor_ptr(sun, n)
        return sun, 3

    def sky_radiance(self, camera, view_ray, sun_direction, shadow_length=None,
                     luminance=False, stream=None):
        """-> (radiance (n, 3), transmittance (n, 3)) tensors."""
        import torch
        n = camera.numel() // 3
        sun, stride = self._sun(sun_direction, n)
        out = torch.empty((n, 3), device=camera.device, dtype=torch.float32)
        tr = torch.empty_like(out)
        _check(lib().atmo_sky_radiance(self._h, _tensor_ptr(camera, n), _tensor_ptr(view_ray, n),
                                       _tensor_ptr(shadow_length), _tensor_ptr(sun), stride, n,
                                       int(bool(luminance)), out.data_ptr(), tr.data_ptr(),
                                       _stream_ptr(stream)))
        return out, tr

    def sky_radiance_to_point(self, camera, point, sun_direction, shadow_length=None,
                              luminance=False, stream=None):
        import torch
        n = camera.numel() // 3
        sun, stride = self._sun(sun_direction, n)
        out = torch.empty((n, 3), device=camera.device, dtype=torch.float32)
        tr = torch.empty_like(out)
        _check(lib().atmo_sky_radiance_to_point(
            self._h, _tensor_ptr(camera, n), _tensor_ptr(point, n), _tensor_ptr(shadow_length),
            _tensor_ptr(sun), stride, n, int(bool(luminance)), out.data_ptr(), tr.data_ptr(),
            _stream_ptr(stream)))
        return out, tr

    def sun_and_sky_irradiance(self, point, normal, sun_direction, luminance=False,
                               stream=None):
        """-> (sun irradiance (n, 3), sky irradiance (n, 3))."""
        import torch
        n = point.numel() // 3
        sun, stride = self._sun(sun_direction, n)
        out = torch.empty((n, 3), device=point.device, dtype=torch.float32)
        sky = torch.empty_like(out)
        _check(lib().atmo_sun_and_sky_irradiance(
            self._h, _tensor_ptr(point, n), _tensor_ptr(normal, n), _tensor_ptr(sun), stride, n,
            int(bool(luminance)), out.data_ptr(), sky.data_ptr(), _stream_ptr(stream)))
        return out, sky

    def read(self, kind):
        """A LUT of the set as a host array (transmittance / irradiance (H, W, 4),
        scattering (R, MU, NU*MU_S, 4))."""
        sh = self._shape()
        if kind in (LUT_TRANSMITTANCE, LUT_IRRADIANCE):
            w, h = ((sh[0], sh[1]) if kind == LUT_TRANSMITTANCE else (sh[6], sh[7]))
            out = np.empty((h, w, 4), np.float32)
        else:
            out = np.empty((sh[2], sh[3], sh[5] * sh[4], 4), np.float32)
        _check(lib().atmo_lut_set_read(self._h, kind, out.ctypes.data_as(C.POINTER(C.c_float)),
                                       out.nbytes))
        return out

    def _shape(self):
        return self._owner_shape

    def solar_radiance(self, luminance=False):
        out = (C.c_double * 3)()
        _check(lib().atmo_solar_radiance(self._h, int(bool(luminance)), out))
        return tuple(out)

    def shade_view(self, view: PinholeView, depth, luminance=False, stream=None):
        """One shading request: -> (sky (H, W, 4), shaded (H, W, 4)) tensors."""
        import torch
        n = view.width * view.height
        if depth.numel() != n:
            raise ValueError("depth needs one value per pixel")
        sky = torch.empty((view.height, view.width, 4), device=depth.device,
                          dtype=torch.float32)
        shaded = torch.empty_like(sky)
        _check(lib().atmo_shade_view(self._h, C.byref(view), _tensor_ptr(depth),
                                     int(bool(luminance)), sky.data_ptr(), shaded.data_ptr(),
                                     _stream_ptr(stream)))
        return sky, shaded


class Server:
    """The serving engine (atmo_server_*): resident LUT sets under an HBM
    budget with LRU eviction, rebuilds batched at pass granularity, shading
    requests on their own streams."""

    QUEUED, RUNNING, DONE, FAILED = range(4)

    def __init__(self, hbm_budget_bytes=0, max_rebuilds_in_flight=0, shade_streams=0,
                 combined=True, admit_window_us=0, pool_max_bytes=0, max_shades_in_flight=0):
        cfg = ServerConfig(hbm_budget_bytes, max_rebuilds_in_flight, shade_streams,
                           int(bool(combined)), admit_window_us, pool_max_bytes,
                           max_shades_in_flight)
        h = C.c_void_p()
        _check(lib().atmo_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._shapes = {}

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.atmo_server_destroy(self._h)
            self._h = None

    __del__ = close

    def submit_rebuild(self, atmosphere, shape=None, orders=4):
        a = Atmosphere.from_buffer_of(atmosphere)
        s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
        t = C.c_uint64()
        _check(lib().atmo_server_submit_rebuild(self._h, C.byref(a), C.byref(s), orders,
                                                C.byref(t)))
        self._shapes[t.value] = s.as_tuple()
        return t.value

    def submit_shade(self, set_id, view, depth, sky, shaded):
        """view: PinholeView; depth (H*W) and sky / shaded (H, W, 4) float32
        CUDA tensors kept alive by the caller until the ticket completes."""
        t = C.c_uint64()
        _check(lib().atmo_server_submit_shade(self._h, set_id, C.byref(view),
                                              _tensor_ptr(depth), _tensor_ptr(sky),
                                              _tensor_ptr(shaded), C.byref(t)))
        return t.value

    def poll(self, ticket) -> TicketInfo:
        info = TicketInfo()
        _check(lib().atmo_server_poll(self._h, ticket, C.byref(info)))
        return info

    def wait(self, ticket, timeout_ms=60000) -> TicketInfo:
        info = TicketInfo()
        _check(lib().atmo_server_wait(self._h, ticket, timeout_ms, C.byref(info)))
        return info

    def cancel(self, ticket):
        """Drops a queued request, or stops a rebuild being built (its memory
        returns to the budget); the ticket then fails with CANCELLED."""
        _check(lib().atmo_server_cancel(self._h, ticket))

    def release_ticket(self, ticket):
        _check(lib().atmo_server_release_ticket(self._h, ticket))

    def lut_set(self, set_id) -> LutSet:
        h = C.c_void_p()
        _check(lib().atmo_server_lut_set(self._h, set_id, C.byref(h)))
        return LutSet(h, self, self._shapes.get(set_id))

    def evict(self, set_id):
        _check(lib().atmo_server_evict(self._h, set_id))

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(lib().atmo_server_get_stats(self._h, C.byref(s)))
        return s


def autotune(atmosphere, shape=None, instances=4) -> Tuning:
    """Times the launchable block shapes of the single- and multiple-scattering
    kernels for `shape` on this GPU and registers the fastest (results are
    bit-identical under every tuning)."""
    t = Tuning()
    s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
    _check(lib().atmo_autotune(C.byref(Atmosphere.from_buffer_of(atmosphere)), C.byref(s),
                               instances, C.byref(t)))
    return t


def set_tuning(shape, tuning=None):
    """Registers (or, with None, clears) a tuning for a LUT shape."""
    s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
    _check(lib().atmo_set_tuning(C.byref(s), C.byref(tuning) if tuning is not None else None))


def get_tuning(shape=None) -> Tuning:
    t = Tuning()
    s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
    _check(lib().atmo_get_tuning(C.byref(s), C.byref(t)))
    return t


def measure_fp32_peak():
    """This GPU's FP32 FMA throughput in TFLOP/s (2 FLOP per FMA)."""
    t = C.c_double()
    _check(lib().atmo_measure_fp32_peak(C.byref(t)))
    return t.value


CHECK_SITES = {1: "shared-memory lookup", 2: "LUT texel", 3: "staged texel",
               4: "line-build row", 5: "line tap", 6: "output texel", 255: "self-test"}


def device_checks(reset=False):
    """The record of the checked build's device-side index checks (after a
    device synchronisation; with reset, cleared): (compiled, failure), where
    compiled is whether this library is the checked build and failure is None
    when every check passed, else (site name, index) of the first failure."""
    compiled, word = C.c_int(), C.c_ulonglong()
    _check(lib().atmo_device_checks(int(bool(reset)), C.byref(compiled), C.byref(word)))
    w = word.value
    if w == 0:
        return bool(compiled.value), None
    return bool(compiled.value), (CHECK_SITES.get(w >> 56, str(w >> 56)), w & ((1 << 56) - 1))


def device_checks_selftest(stream=None):
    """Launches one check that fails by construction (index 5 of 3, no access)."""
    _check(lib().atmo_device_checks_selftest(stream))


def synchronize_stream(stream=None):
    """Waits for the work enqueued on `stream` (None: the default stream)."""
    _check(lib().atmo_synchronize(_stream_ptr(stream)))


class Batch:
    """Many independent atmospheres (uneven LUT shapes and order counts)
    precomputed together; the pass sequence replays as a CUDA graph."""

    def __init__(self, atmospheres, shapes=None, orders=4, combined=True):
        n = len(atmospheres)
        self.n = n
        self._atm = (Atmosphere * n)(*[Atmosphere.from_buffer_of(a) for a in atmospheres])
        if shapes is None:
            shapes = [DEFAULT_SHAPE] * n
        self.shapes = [LutShape.of(s) for s in shapes]
        self._shapes = (LutShape * n)(*self.shapes)
        if isinstance(orders, int):
            orders = [orders] * n
        self.orders = list(orders)
        self._orders = (C.c_uint * n)(*self.orders)
        self.combined = combined
        h = C.c_void_p()
        _check(lib().atmo_batch_create(self._atm, self._shapes, self._orders, n,
                                       int(bool(combined)), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.atmo_batch_destroy(h)
            self._h = None

    def set_atmosphere(self, i, atmosphere):
        a = Atmosphere.from_buffer_of(atmosphere)
        _check(lib().atmo_batch_set_atmosphere(self._h, i, C.byref(a)))

    def run(self, stream=None):
        _check(lib().atmo_batch_run(self._h, _stream_ptr(stream)))

    def save_luts(self, i, directory):
        _check(lib().atmo_batch_save_luts(self._h, i, os.fsencode(directory)))

    def copy_lut(self, i, kind, dst_ptr, nbytes, stream=None):
        """Stream-ordered copy of a LUT into dst (device or pinned host)."""
        _check(lib().atmo_batch_copy_lut(self._h, i, kind, dst_ptr, nbytes,
                                         _stream_ptr(stream)))

    def lut_set(self, i) -> "LutSet":
        h = C.c_void_p()
        _check(lib().atmo_batch_lut_set(self._h, i, C.byref(h)))
        return LutSet(h, self, self.shapes[i].as_tuple())

    def kernel_count(self):
        c = C.c_uint()
        _check(lib().atmo_batch_kernel_count(self._h, C.byref(c)))
        return c.value

    PASS_NAMES = ("tables", "transmittance", "direct_irradiance", "single_scattering",
                  "scattering_density", "indirect_irradiance", "multiple_scattering",
                  "to_half")

    def time_passes(self, stream=None):
        """[(pass name, order, ms)] of one non-graph run, CUDA-event timed."""
        cap = 4096
        ms, ps, od = (C.c_float * cap)(), (C.c_int * cap)(), (C.c_int * cap)()
        n = C.c_uint()
        _check(lib().atmo_batch_time_passes(self._h, _stream_ptr(stream), cap, ms, ps, od,
                                            C.byref(n)))
        return [(self.PASS_NAMES[ps[i]], od[i], ms[i]) for i in range(min(n.value, cap))]

    def lut_view(self, i, kind) -> LutView:
        v = LutView()
        _check(lib().atmo_batch_get_lut(self._h, i, kind, C.byref(v)))
        return v

    def read(self, i, kind):
        v = self.lut_view(i, kind)
        out = np.empty((v.depth, v.height, v.width, 4), np.float32)
        _check(lib().atmo_batch_read_lut(self._h, i, kind,
                                         out.ctypes.data_as(C.POINTER(C.c_float)), out.nbytes))
        return out if v.depth > 1 else out[0]


PASS_SCATTERING_DENSITY, PASS_INDIRECT_IRRADIANCE, PASS_MULTIPLE_SCATTERING = 4, 5, 6


def run_pass(atmosphere, shape, pass_kind, order, path=PATH_FAST, stream=None, **buffers):
    """One pass of Model::Precompute's order loop (atmosphere/model.cc:1137-1211)
    on caller-owned float32 RGBA device LUTs (keyword arguments named as the
    fields of atmo_pass_buffers: CUDA tensors or device pointers; the pass
    reads and writes them as atmo_run_pass documents).  Synchronous."""
    a = Atmosphere.from_buffer_of(atmosphere)
    s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
    ptr = lambda t: None if t is None else (t if isinstance(t, int) else t.data_ptr())  # noqa
    unknown = set(buffers) - {n for n, _ in PassBuffers._fields_}
    if unknown:
        raise TypeError("unknown buffers: %s" % sorted(unknown))
    b = PassBuffers(*[ptr(buffers.get(n)) for n, _ in PassBuffers._fields_])
    _check(lib().atmo_run_pass(C.byref(a), C.byref(s), pass_kind, order, path, C.byref(b),
                               _stream_ptr(stream)))


def precompute(atmosphere, shape, num_scattering_orders, transmittance, scattering, single_mie,
               irradiance, lum=None, blend=False, combined=True, path=PATH_FAST, stream=None):
    """One Model::Precompute group (atmosphere/model.cc:1048-1215) into
    caller-owned float32 RGBA device buffers (device pointers as ints, or
    objects with data_ptr())."""
    a = Atmosphere.from_buffer_of(atmosphere)
    s = LutShape.of(shape) or LutShape(*DEFAULT_SHAPE)
    lum_arr = None
    if lum is not None:
        lum_arr = (C.c_float * 9)(*[float(x) for x in np.asarray(lum).reshape(9)])
    ptr = lambda t: None if t is None else (t if isinstance(t, int) else t.data_ptr())  # noqa
    _check(lib().atmo_precompute(C.byref(a), C.byref(s), num_scattering_orders, lum_arr,
                                 int(bool(blend)), int(bool(combined)), path, ptr(transmittance),
                                 ptr(scattering), ptr(single_mie), ptr(irradiance),
                                 _stream_ptr(stream)))
