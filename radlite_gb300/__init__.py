"""GB300-native line raytrace for RADLite models (drop-in for the RADlite raytrace step).

The compute path is the in-tree CUDA library ``_lib/librlgpu.so`` (sm_103a kernels behind
the C ABI of ``include/rlgpu.h``). This module is a thin ctypes binding over that ABI that
mirrors the reference's entry points:

  run_dir(dir)                    the RADlite executable run in a working directory
                                  (RADLITE/main.F:26-71): writes linespectrum_<mol>.dat
  Model.calc_line_spectrum(iline) calc_line_spectrum (RADLITE/telescope.F:1465-1654):
                                  F_nu at 1 pc over the passband (spec_flux_observer)
  Model.line_image(iline)         the circular image imcir_int (telescope.F:339-631)

There is no CPU fallback: importing works without a GPU, but every call that computes
needs the built library and a CUDA device and raises otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librlgpu.so")
EXE_PATH = os.path.join(_HERE, "_lib", "RADlite_gpu")

RL_FP32, RL_FP64 = 0, 1


class RLError(RuntimeError):
    pass


class Stats(C.Structure):
    _fields_ = [("steps", C.c_ulonglong), ("integrated", C.c_ulonglong), ("node_visits", C.c_ulonglong),
                ("ray_channels", C.c_ulonglong), ("geometry_ms", C.c_double), ("walk_ms", C.c_double),
                ("reduce_ms", C.c_double), ("upload_ms", C.c_double), ("total_ms", C.c_double),
                ("nrays", C.c_int), ("nfr", C.c_int), ("kmax", C.c_int), ("nlines", C.c_int),
                ("h2d_bytes", C.c_ulonglong), ("d2h_bytes", C.c_ulonglong), ("node_passes", C.c_ulonglong),
                ("packed_passes", C.c_ulonglong), ("empty_steps", C.c_ulonglong),
                ("refined_passes", C.c_ulonglong), ("sub_steps", C.c_ulonglong),
                ("refined_channels", C.c_ulonglong), ("overshoots", C.c_ulonglong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ModelInfo(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nr", "nth", "nlev", "nlines_mol", "nlines_spec", "ilinestart", "nfr",
                                       "nphi", "dbdr", "nrrayextra", "nrays", "nrings", "outer_bc", "starpump",
                                       "line_dust", "precision")] + \
               [(n, C.c_double) for n in ("incl_deg", "vmax", "dv", "rstar", "aksmax")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class ModelArrays(C.Structure):
    _fields_ = [("nr", C.c_int), ("nth", C.c_int), ("radius", _D), ("theta", _D), ("rho", _D), ("abund", _D),
                ("width", _D), ("vel", _D), ("nlev", C.c_int), ("pop", _D), ("nlines_mol", C.c_int),
                ("lev_up", _I), ("lev_low", _I), ("aud", _D), ("energy_cm", _D), ("gdeg", _D),
                ("umass", C.c_double), ("line_dust", C.c_int), ("ncont", C.c_int), ("freq", _D),
                ("dust_rho", _D), ("dust_temp", _D), ("kappa_abs", _D), ("kappa_scat", _D),
                ("rstar", C.c_double), ("star_flux_1pc", _D), ("outer_bc", C.c_int), ("incl_deg", C.c_double),
                ("nphi", C.c_int), ("dbdr", C.c_int), ("nrrayextra", C.c_int), ("vmax", C.c_double),
                ("dv", C.c_double), ("radvelo", C.c_double), ("ilinestart", C.c_int), ("nlines_spec", C.c_int),
                ("molname", C.c_char_p)]


class PosvelSpec(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("szimx", C.c_double), ("szimy", C.c_double),
                ("phioff", C.c_double), ("xoff", C.c_double), ("yoff", C.c_double), ("addstar", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GenspecLines(C.Structure):
    _fields_ = [("nlines", C.c_int), ("npts", _I), ("vel", _D), ("flux", _D), ("freq", _D), ("maxnumpoints", _I)]


class GenspecParams(C.Structure):
    _fields_ = [("obsres", C.c_double), ("vsampling", C.c_double), ("dist", C.c_double)]


EXPORTS = ["rl_create", "rl_destroy", "rl_last_error", "rl_load_dir", "rl_load_arrays", "rl_model_free",
           "rl_model_get_info", "rl_set_camera", "rl_set_precision", "rl_set_checks", "rl_line_spectrum",
           "rl_spectra",
           "rl_line_image", "rl_run_dir", "rl_debug_trajectory", "rl_measure_peaks",
           "rl_batch_create", "rl_batch_destroy", "rl_batch_add", "rl_batch_set_memory", "rl_batch_set_tiles",
           "rl_batch_get_tiles", "rl_batch_autotune", "rl_batch_use_graph", "rl_batch_flux_size",
           "rl_batch_job_info", "rl_batch_job_masing", "rl_batch_run", "rl_batch_waves", "rl_run_manifest",
           "rl_diff_create", "rl_diff_destroy", "rl_diff_info", "rl_diff_set_checkpoint", "rl_diff_forward",
           "rl_diff_backward", "rl_diff_batch_create", "rl_diff_batch_destroy", "rl_diff_batch_add",
           "rl_diff_batch_use_graph", "rl_diff_batch_buffers", "rl_diff_batch_layout", "rl_diff_batch_forward",
           "rl_diff_batch_backward",
           "rl_image_to_spectrum_noalloc", "rl_set_posvel", "rl_get_posvel", "rl_posvel",
           "rl_line_image_mask", "rl_image_rows", "rl_line_masing", "rl_run_dir_ex", "rl_gen_spec_size", "rl_gen_spec",
           "rl_model_checksum"]

_lib = None


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RLError(f"{LIB_PATH} is missing: build it with radlite_gb300.build.build() (no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.rl_create.argtypes = [C.POINTER(vp), C.c_int]
        L.rl_destroy.argtypes = [vp]
        L.rl_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.rl_load_dir.argtypes = [vp, C.c_char_p, C.POINTER(vp)]
        L.rl_load_arrays.argtypes = [vp, C.POINTER(ModelArrays), C.POINTER(vp)]
        L.rl_model_free.argtypes = [vp]
        L.rl_model_get_info.argtypes = [vp, C.POINTER(ModelInfo)]
        L.rl_model_checksum.argtypes = [vp, C.POINTER(C.c_ulonglong)]
        L.rl_set_camera.argtypes = [vp, C.c_double, C.c_int, C.c_int, C.c_int]
        L.rl_set_precision.argtypes = [vp, C.c_int]
        L.rl_set_checks.argtypes = [vp, C.c_int]
        L.rl_line_spectrum.argtypes = [vp, C.c_int, _D, _D, C.POINTER(Stats)]
        L.rl_spectra.argtypes = [vp, C.c_int, C.c_int, _D, C.POINTER(Stats)]
        L.rl_line_image.argtypes = [vp, C.c_int, _D, C.POINTER(Stats)]
        L.rl_run_dir.argtypes = [C.c_char_p, C.c_int, C.POINTER(Stats)]
        L.rl_run_dir_ex.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(Stats)]
        L.rl_line_image_mask.argtypes = [vp, C.c_int, _D, C.POINTER(C.c_ubyte), C.POINTER(Stats)]
        L.rl_image_rows.argtypes = [vp, C.c_int, C.c_int, C.c_int, _I, _D, _D, C.POINTER(Stats)]
        L.rl_set_posvel.argtypes = [vp, C.POINTER(PosvelSpec)]
        L.rl_gen_spec_size.argtypes = [C.POINTER(GenspecLines), C.POINTER(GenspecParams), C.POINTER(C.c_longlong)]
        L.rl_gen_spec.argtypes = [vp, C.POINTER(GenspecLines), C.POINTER(GenspecParams)] + [_D] * 5 + [C.POINTER(Stats)]
        L.rl_get_posvel.argtypes = [vp, C.POINTER(PosvelSpec)]
        L.rl_posvel.argtypes = [vp, C.c_int, C.c_int, _D, _D, C.POINTER(Stats)]
        L.rl_debug_trajectory.argtypes = [vp, C.c_int, C.c_int, _D, _D, _D, _D, _D, _I, _I, _I]
        L.rl_measure_peaks.argtypes = [vp, _D, _D]
        L.rl_batch_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
        L.rl_batch_destroy.argtypes = [vp]
        L.rl_batch_add.argtypes = [vp, vp, C.c_int, C.c_int]
        L.rl_batch_set_memory.argtypes = [vp, C.c_double]
        L.rl_batch_set_tiles.argtypes = [vp, C.c_int, C.c_int]
        L.rl_batch_get_tiles.argtypes = [vp, _I, _I]
        L.rl_batch_autotune.argtypes = [vp, C.c_int, _I, _I, _D]
        L.rl_batch_use_graph.argtypes = [vp, C.c_int]
        L.rl_batch_flux_size.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.rl_batch_job_info.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong), _I, _I]
        L.rl_batch_run.argtypes = [vp, _D, C.POINTER(Stats)]
        L.rl_batch_job_masing.argtypes = [vp, C.c_int, _I]
        L.rl_batch_waves.argtypes = [vp, _I]
        L.rl_run_manifest.argtypes = [C.c_char_p, C.c_int, C.POINTER(Stats)]
        L.rl_diff_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]
        L.rl_diff_destroy.argtypes = [vp]
        L.rl_diff_info.argtypes = [vp, _I, _I, _I, _I]
        L.rl_diff_set_checkpoint.argtypes = [vp, C.c_int]
        L.rl_diff_batch_create.argtypes = [vp, C.POINTER(vp)]
        L.rl_diff_batch_destroy.argtypes = [vp]
        L.rl_diff_batch_add.argtypes = [vp, vp]
        L.rl_diff_batch_use_graph.argtypes = [vp, C.c_int]
        L.rl_diff_batch_buffers.argtypes = [vp] + [C.POINTER(vp)] * 8 + [C.POINTER(C.c_longlong)] * 2
        L.rl_diff_batch_layout.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.rl_diff_batch_forward.argtypes = [vp, C.POINTER(Stats)]
        L.rl_diff_batch_backward.argtypes = [vp, C.POINTER(Stats)]
        L.rl_diff_forward.argtypes = [vp, vp, vp, vp, vp, C.POINTER(Stats)]
        L.rl_diff_backward.argtypes = [vp, vp, vp, vp, vp, C.POINTER(Stats)]
        L.rl_image_to_spectrum_noalloc.argtypes = [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                   vp, vp, C.c_double, vp]
        _lib = L
    return _lib


def _err(ctx=None) -> str:
    buf = C.create_string_buffer(2048)
    lib().rl_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc, ctx=None):
    if rc < 0:
        raise RLError(_err(ctx))
    return rc


def _dp(a):
    return a.ctypes.data_as(_D)


class Context:
    """One CUDA device with its stream (rl_ctx)."""

    def __init__(self, device: int = 0):
        self.h = C.c_void_p()
        self._children = []   # weak references to the models, batches and diffs made on it
        _check(lib().rl_create(C.byref(self.h), device))

    def _adopt(self, obj, rank: int):
        """Record an object that must be released before the context (lower rank first)."""
        self._children.append((rank, weakref.ref(obj)))

    def close(self):
        """Release every model, batch and differentiable handle still open on this context,
        then the context itself (the library's handles must not outlive their context)."""
        if self.h:
            for _, ref in sorted(self._children, key=lambda t: t[0]):
                obj = ref()
                if obj is not None:
                    try:
                        obj.free() if hasattr(obj, "free") else obj.close()
                    except Exception:
                        pass
            self._children = []
            lib().rl_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def gen_spec(self, lines, obsres: float, vsampling: float, dist: float, stats: bool = False) -> dict:
        """The numerical core of pyradlite's RadliteSpectrum.gen_spec on the GPU: `lines` is a
        list of dicts with "vel" (ascending, km/s), "flux" (F_nu at 1 pc), "freq" (Hz) and
        "maxnumpoints"; returns wavelength [micron], frequency [Hz], spectrum, emission and
        continuum [Jy at dist pc]."""
        vel = np.ascontiguousarray(np.concatenate([np.asarray(d["vel"], dtype=np.float64) for d in lines]))
        flux = np.ascontiguousarray(np.concatenate([np.asarray(d["flux"], dtype=np.float64) for d in lines]))
        npts = np.array([len(d["vel"]) for d in lines], dtype=np.int32)
        freq = np.array([d["freq"] for d in lines], dtype=np.float64)
        mx = np.array([d["maxnumpoints"] for d in lines], dtype=np.int32)
        L = GenspecLines(len(lines), npts.ctypes.data_as(_I), _dp(vel), _dp(flux), _dp(freq), mx.ctypes.data_as(_I))
        P = GenspecParams(obsres, vsampling, dist)
        n = C.c_longlong()
        _check(lib().rl_gen_spec_size(C.byref(L), C.byref(P), C.byref(n)))
        out = {k: np.zeros(n.value) for k in ("wavelength", "frequency", "spectrum", "emission", "continuum")}
        st = Stats()
        _check(lib().rl_gen_spec(self.h, C.byref(L), C.byref(P), *(_dp(out[k]) for k in
                                 ("wavelength", "frequency", "spectrum", "emission", "continuum")), C.byref(st)), self.h)
        if stats:
            out["stats"] = st.as_dict()
        return out

    def measure_peaks(self) -> dict:
        """Measured FP32 FFMA and MUFU ex2 throughput of the device (lane ops per second)."""
        a, b = C.c_double(), C.c_double()
        _check(lib().rl_measure_peaks(self.h, C.byref(a), C.byref(b)), self.h)
        return {"ffma_per_s": a.value, "ex2_per_s": b.value}

    def load_dir(self, path: str) -> "Model":
        h = C.c_void_p()
        _check(lib().rl_load_dir(self.h, os.fsencode(path), C.byref(h)), self.h)
        return Model(self, h)

    def load_arrays(self, arrays: dict, camera: dict) -> "Model":
        """Model from in-memory arrays (the content of the input files, see synth.model_arrays)."""
        keep = []

        def arr(x, dt=np.float64):
            a = np.ascontiguousarray(x, dtype=dt)
            keep.append(a)
            return a.ctypes.data_as(_D if dt == np.float64 else _I)

        f = arrays
        cell = lambda a: np.asarray(a).T.ravel()   # [nt, nr] -> (ir-1)*nth + (it-1)
        nt, nr = f["rho"].shape
        pop = f["pop"].transpose(2, 1, 0).reshape(nr * nt, -1)
        vel = np.stack([cell(f["vel"][0]), cell(f["vel"][1]), cell(f["vel"][2])], axis=1)
        lines = f["lines"]
        a = ModelArrays()
        a.nr, a.nth = nr, nt
        a.radius, a.theta = arr(f["r"]), arr(f["theta"])
        a.rho, a.abund, a.width = arr(cell(f["rho"])), arr(cell(f["abund"])), arr(cell(f["width"]))
        a.vel = arr(vel)
        a.nlev = pop.shape[1]
        a.pop = arr(pop)
        a.nlines_mol = len(lines)
        a.lev_up = arr([u for u, _, _ in lines], np.int32)
        a.lev_low = arr([l for _, l, _ in lines], np.int32)
        a.aud = arr([float(f"{A:.3e}") for _, _, A in lines])
        a.energy_cm = arr(np.round(f["E"], 4))
        a.gdeg = arr(f["g"])
        a.umass = 2.3
        a.line_dust = 1
        a.ncont = len(f["freq"])
        a.freq = arr(f["freq"])
        a.dust_rho, a.dust_temp = arr(cell(f["dust_rho"])), arr(cell(f["dust_temp"]))
        a.kappa_abs, a.kappa_scat = arr(f["kappa_abs"]), arr(f["kappa_scat"])
        a.rstar = f["rstar"]
        a.star_flux_1pc = arr(f["star_flux_1pc"]) if camera.get("starpump", 1) else C.cast(None, _D)
        a.outer_bc = camera.get("outer_bc", 0)
        a.incl_deg = camera["incl_deg"]
        a.nphi, a.dbdr, a.nrrayextra = camera["nphi"], camera["dbdr"], camera["nrrayextra"]
        a.vmax, a.dv, a.radvelo = camera["vmax"], camera["dv"], camera.get("radvelo", 0.0)
        a.ilinestart, a.nlines_spec = camera["ilinestart"], camera["nlines"]
        a.molname = camera.get("molname", "moldata").encode()
        h = C.c_void_p()
        _check(lib().rl_load_arrays(self.h, C.byref(a), C.byref(h)), self.h)
        return Model(self, h)


class Model:
    """A loaded RADLite model on the GPU (rl_model)."""

    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h
        if ctx is not None:
            ctx._adopt(self, 3)

    def free(self):
        if self.h:
            lib().rl_model_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def checksum(self) -> int:
        """Hash of everything the model holds from its inputs."""
        v = C.c_ulonglong()
        _check(lib().rl_model_checksum(self.h, C.byref(v)), self._ch)
        return v.value

    def info(self) -> dict:
        i = ModelInfo()
        _check(lib().rl_model_get_info(self.h, C.byref(i)))
        return i.as_dict()

    @property
    def _ch(self):
        return self.ctx.h if self.ctx is not None else None

    def set_camera(self, incl_deg, nphi, dbdr, nrrayextra):
        _check(lib().rl_set_camera(self.h, incl_deg, nphi, dbdr, nrrayextra), self._ch)

    def set_precision(self, precision: int):
        _check(lib().rl_set_precision(self.h, precision), self._ch)

    def set_checks(self, overshoot: bool = True):
        """Take the reference's overshoot test on every step of this model's line renders
        and count the steps that fail it (stats["overshoots"]); results are unchanged."""
        _check(lib().rl_set_checks(self.h, CHECK_OVERSHOOT if overshoot else 0), self._ch)

    def calc_line_spectrum(self, iline: int, stats: bool = False):
        """F_nu at 1 pc over the passband of line `iline` (1-based, moldata.dat order)."""
        n = self.info()["nfr"]
        flux, velo = np.zeros(n), np.zeros(n)
        st = Stats()
        _check(lib().rl_line_spectrum(self.h, iline, _dp(flux), _dp(velo), C.byref(st)), self._ch)
        return (flux, velo, st.as_dict()) if stats else (flux, velo)

    def spectra(self, iline0: int, nlines: int, stats: bool = False):
        n = self.info()["nfr"]
        flux = np.zeros((nlines, n))
        st = Stats()
        _check(lib().rl_spectra(self.h, iline0, nlines, _dp(flux), C.byref(st)), self._ch)
        return (flux, st.as_dict()) if stats else flux

    def line_image(self, iline: int, mask: bool = False):
        """Circular image [nrays, nfr] (imcir_int); with mask=True also the integration mask
        (imcir_cmask: 1 = channel 1 or inside the ray's velocity window)."""
        info = self.info()
        img = np.zeros((info["nrays"], info["nfr"]))
        st = Stats()
        if not mask:
            _check(lib().rl_line_image(self.h, iline, _dp(img), C.byref(st)), self._ch)
            return img
        msk = np.zeros((info["nrays"], info["nfr"]), dtype=np.uint8)
        _check(lib().rl_line_image_mask(self.h, iline, _dp(img), msk.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                        C.byref(st)), self._ch)
        return img, msk

    def image_rows(self, iline0: int, nlines: int, rays, stats: bool = False):
        """Lines iline0.. in one launch: their spectra [nlines, nfr] and the image rows of the
        chosen rays [nlines, len(rays), nfr] (a ray sample of line_image's images)."""
        n = self.info()["nfr"]
        r = np.ascontiguousarray(rays, dtype=np.int32)
        flux = np.zeros((nlines, n))
        rows = np.zeros((nlines, len(r), n))
        st = Stats()
        _check(lib().rl_image_rows(self.h, iline0, nlines, len(r), r.ctypes.data_as(_I), _dp(flux), _dp(rows),
                                   C.byref(st)), self._ch)
        return (flux, rows, st.as_dict()) if stats else (flux, rows)

    def masing(self, iline: int) -> bool:
        """Whether the last render of line `iline` met the reference's masing test (a line
        opacity x segment length below -0.01, telescope.F:4291-4297)."""
        d = C.c_int()
        _check(lib().rl_line_masing(self.h, iline, C.byref(d)), self._ch)
        return bool(d.value)

    def set_posvel(self, nx: int, ny: int, szimx: float, szimy: float, phioff: float = 0.0, xoff: float = 0.0,
                   yoff: float = 0.0, addstar: int = 1):
        """The rectangular image of linespectrum.inp command 2: nx x ny pixels (even) over a
        full image size szimx x szimy [cm], rotation phioff [rad], offsets [cm]."""
        sp = PosvelSpec(nx, ny, szimx, szimy, phioff, xoff, yoff, addstar)
        _check(lib().rl_set_posvel(self.h, C.byref(sp)), self._ch)

    def posvel_spec(self) -> dict:
        sp = PosvelSpec()
        _check(lib().rl_get_posvel(self.h, C.byref(sp)), self._ch)
        return sp.as_dict()

    def posvel(self, iline0: int, nlines: int = 1, stats: bool = False):
        """Intensity and optical-depth cubes [nlines, nfr, ny, nx] of the position-velocity
        image (imrec_int, imrec_tau)."""
        sp = self.posvel_spec()
        shape = (nlines, self.info()["nfr"], sp["ny"], sp["nx"])
        I, tau = np.zeros(shape), np.zeros(shape)
        st = Stats()
        _check(lib().rl_posvel(self.h, iline0, nlines, _dp(I), _dp(tau), C.byref(st)), self._ch)
        return (I, tau, st.as_dict()) if stats else (I, tau)

    def trajectory(self, iray: int, cap: int = 8192) -> dict:
        out = {k: np.zeros(cap) for k in ("s", "r", "theta", "mu", "dvmu")}
        iv = {k: np.zeros(cap, dtype=np.int32) for k in ("icr", "ir", "it")}
        n = _check(lib().rl_debug_trajectory(self.h, iray, cap, *(_dp(out[k]) for k in ("s", "r", "theta", "mu", "dvmu")),
                                             *(iv[k].ctypes.data_as(_I) for k in ("icr", "ir", "it"))), self._ch)
        n = min(n, cap)
        res = {k: v[:n] for k, v in out.items()}
        res.update({k: v[:n] for k, v in iv.items()})
        return res


class Batch:
    """Many (model, camera, line range) jobs rendered by one launch sequence (rl_batch).

    Replaces a driver loop over model directories: every job's inputs stay on the device,
    the geometry, walk and reduction of all jobs run as one launch each per memory wave,
    and the sequence is replayed from a CUDA graph."""

    def __init__(self, ctx: Context, precision: int = 0):
        self.ctx = ctx
        self.h = C.c_void_p()
        self.models = []
        _check(lib().rl_batch_create(ctx.h, precision, C.byref(self.h)), ctx.h)
        ctx._adopt(self, 1)

    def close(self):
        if self.h:
            lib().rl_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, model: "Model", iline0: int, nlines: int) -> int:
        """Queue lines iline0 .. iline0+nlines-1 of `model` at its current camera."""
        self.models.append(model)   # the batch reads the model's device grid
        return _check(lib().rl_batch_add(self.h, model.h, iline0, nlines), self.ctx.h)

    def set_memory(self, nbytes: float):
        _check(lib().rl_batch_set_memory(self.h, float(nbytes)), self.ctx.h)

    def set_tiles(self, lines_per_item: int, channel_slots: int):
        _check(lib().rl_batch_set_tiles(self.h, lines_per_item, channel_slots), self.ctx.h)

    def tiles(self) -> tuple:
        g, c = C.c_int(), C.c_int()
        _check(lib().rl_batch_get_tiles(self.h, C.byref(g), C.byref(c)), self.ctx.h)
        return g.value, c.value

    def autotune(self, sample_stride: int = 8) -> dict:
        g, c, ms = C.c_int(), C.c_int(), C.c_double()
        _check(lib().rl_batch_autotune(self.h, sample_stride, C.byref(g), C.byref(c), C.byref(ms)), self.ctx.h)
        return {"lines_per_item": g.value, "channel_slots": c.value, "sample_ms": ms.value}

    def use_graph(self, enable: bool):
        _check(lib().rl_batch_use_graph(self.h, int(bool(enable))), self.ctx.h)

    def waves(self) -> int:
        n = C.c_int()
        _check(lib().rl_batch_waves(self.h, C.byref(n)), self.ctx.h)
        return n.value

    def run(self, stats: bool = False):
        """Spectra of every job: a list of [nlines, nfr] arrays in job order."""
        n = C.c_longlong()
        _check(lib().rl_batch_flux_size(self.h, C.byref(n)), self.ctx.h)
        flux = np.zeros(n.value)
        st = Stats()
        _check(lib().rl_batch_run(self.h, _dp(flux), C.byref(st)), self.ctx.h)
        out = []
        for j in range(len(self.models)):
            off, nl, nfr = C.c_longlong(), C.c_int(), C.c_int()
            _check(lib().rl_batch_job_info(self.h, j, C.byref(off), C.byref(nl), C.byref(nfr)), self.ctx.h)
            out.append(flux[off.value:off.value + nl.value * nfr.value].reshape(nl.value, nfr.value))
        return (out, st.as_dict()) if stats else out

    def masing(self, job: int) -> np.ndarray:
        """Per line of job `job`: whether the last run met the reference's masing test."""
        off, nl, nfr = C.c_longlong(), C.c_int(), C.c_int()
        _check(lib().rl_batch_job_info(self.h, job, C.byref(off), C.byref(nl), C.byref(nfr)), self.ctx.h)
        d = np.zeros(nl.value, dtype=np.int32)
        _check(lib().rl_batch_job_masing(self.h, job, d.ctypes.data_as(_I)), self.ctx.h)
        return d.astype(bool)


class Diff:
    """Differentiable spectra of one model (rl_diff): F_nu[lines, channels] as a function of
    per-cell ln T, ln X (abundance) and line width b [km/s], cells in the library order
    (ir-1)*nth + (it-1). Arrays are float64 CUDA tensors (torch) on the context's device."""

    def __init__(self, model: "Model", iline0: int, nlines: int, precision: int = RL_FP32):
        self.model = model
        self.h = C.c_void_p()
        _check(lib().rl_diff_create(model.h, iline0, nlines, precision, C.byref(self.h)), model._ch)
        if model.ctx is not None:
            model.ctx._adopt(self, 1)
        nc, nl, nf, nr = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().rl_diff_info(self.h, C.byref(nc), C.byref(nl), C.byref(nf), C.byref(nr)))
        self.ncell, self.nlines, self.nfr, self.nrays = nc.value, nl.value, nf.value, nr.value
        self.version = 0

    def set_checkpoint(self, every: int):
        """How the adjoint walks each ray: 0 (default) the gradient sweep in walk order;
        1 or 32 the reverse sweep with intensities stored every node or every 32 nodes."""
        _check(lib().rl_diff_set_checkpoint(self.h, every), self.model._ch)

    def close(self):
        if self.h:
            lib().rl_diff_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _dev(t):
        import torch
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise RLError("Diff takes contiguous float64 CUDA tensors")
        return t

    def forward(self, lnT, lnX, width, stats: bool = False):
        import torch
        for t in (lnT, lnX, width):
            self._dev(t)
            if t.numel() != self.ncell:
                raise RLError(f"expected {self.ncell} cells, got {t.numel()}")
        flux = torch.empty((self.nlines, self.nfr), dtype=torch.float64, device=lnT.device)
        torch.cuda.current_stream(lnT.device).synchronize()
        st = Stats()
        _check(lib().rl_diff_forward(self.h, lnT.data_ptr(), lnX.data_ptr(), width.data_ptr(), flux.data_ptr(),
                                     C.byref(st)), self.model._ch)
        self.version += 1
        return (flux, st.as_dict()) if stats else flux

    def backward(self, gflux, stats: bool = False):
        import torch
        gflux = self._dev(gflux.contiguous())
        g = [torch.empty(self.ncell, dtype=torch.float64, device=gflux.device) for _ in range(3)]
        torch.cuda.current_stream(gflux.device).synchronize()
        st = Stats()
        _check(lib().rl_diff_backward(self.h, gflux.data_ptr(), g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                      C.byref(st)), self.model._ch)
        return (tuple(g), st.as_dict()) if stats else tuple(g)


class _DevArray:
    """A float64 device buffer owned by the library, exposed through
    __cuda_array_interface__ so that torch.as_tensor wraps it without a copy."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3,
                                         "strides": None}


class DiffBatch:
    """Many Diff models rendered by one forward and one adjoint launch sequence, each
    replayed from a CUDA graph (rl_diff_batch). The parameter, spectrum and gradient
    buffers belong to the batch; `tensors()` returns torch views of them per model."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = C.c_void_p()
        self.diffs = []
        _check(lib().rl_diff_batch_create(ctx.h, C.byref(self.h)), ctx.h)
        ctx._adopt(self, 0)
        self._views = None

    def close(self):
        if self.h:
            lib().rl_diff_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, diff: Diff) -> int:
        self.diffs.append(diff)
        self._views = None
        return _check(lib().rl_diff_batch_add(self.h, diff.h), self.ctx.h)

    def use_graph(self, enable: bool):
        _check(lib().rl_diff_batch_use_graph(self.h, int(bool(enable))), self.ctx.h)

    def tensors(self) -> dict:
        """torch views of the batch buffers: whole arrays ('lnT', ..., 'g_width') and per-model
        slices ('models': [{'lnT', 'lnX', 'width', 'flux' [nl, nfr], 'gflux', 'g_lnT', ...}])."""
        import torch
        if self._views is not None:
            return self._views
        ptr = [C.c_void_p() for _ in range(8)]
        nc, nf = C.c_longlong(), C.c_longlong()
        _check(lib().rl_diff_batch_buffers(self.h, *(C.byref(p) for p in ptr), C.byref(nc), C.byref(nf)),
               self.ctx.h)
        names = ("lnT", "lnX", "width", "flux", "gflux", "g_lnT", "g_lnX", "g_width")
        sizes = (nc.value, nc.value, nc.value, nf.value, nf.value, nc.value, nc.value, nc.value)
        whole = {k: torch.as_tensor(_DevArray(p.value, n), device="cuda") for k, p, n in zip(names, ptr, sizes)}
        models = []
        for j, d in enumerate(self.diffs):
            co, fo = C.c_longlong(), C.c_longlong()
            _check(lib().rl_diff_batch_layout(self.h, j, C.byref(co), C.byref(fo)), self.ctx.h)
            c0, f0 = co.value, fo.value
            v = {k: whole[k][c0:c0 + d.ncell] for k in ("lnT", "lnX", "width", "g_lnT", "g_lnX", "g_width")}
            for k in ("flux", "gflux"):
                v[k] = whole[k][f0:f0 + d.nlines * d.nfr].view(d.nlines, d.nfr)
            models.append(v)
        whole["models"] = models
        self._views = whole
        return whole

    def forward(self, stats: bool = False):
        import torch
        torch.cuda.current_stream().synchronize()
        st = Stats()
        _check(lib().rl_diff_batch_forward(self.h, C.byref(st)), self.ctx.h)
        return st.as_dict() if stats else None

    def backward(self, stats: bool = False):
        import torch
        torch.cuda.current_stream().synchronize()
        st = Stats()
        _check(lib().rl_diff_batch_backward(self.h, C.byref(st)), self.ctx.h)
        return st.as_dict() if stats else None


def _raytrace_function():
    import torch

    class RaytraceFunction(torch.autograd.Function):
        """spectra = raytrace(ln T, ln X, width); backward by the adjoint walk."""

        @staticmethod
        def forward(ctx, lnT, lnX, width, diff):
            flux = diff.forward(lnT.contiguous(), lnX.contiguous(), width.contiguous())
            ctx.diff, ctx.version = diff, diff.version
            ctx.save_for_backward(lnT, lnX, width)
            return flux

        @staticmethod
        def backward(ctx, gflux):
            diff = ctx.diff
            if diff.version != ctx.version:       # another forward ran since: restore this point
                lnT, lnX, width = ctx.saved_tensors
                diff.forward(lnT.contiguous(), lnX.contiguous(), width.contiguous())
            gT, gX, gb = diff.backward(gflux)
            return gT, gX, gb, None

    return RaytraceFunction


_RF = None


def raytrace(diff: Diff, lnT, lnX, width):
    """Differentiable spectra [nlines, nfr] of `diff` (torch autograd through the adjoint)."""
    global _RF
    if _RF is None:
        _RF = _raytrace_function()
    return _RF.apply(lnT, lnX, width, diff)


def load_dir_host(path: str) -> "Model":
    """Parse a model directory without a device (host-side checks of the input files)."""
    h = C.c_void_p()
    _check(lib().rl_load_dir(None, os.fsencode(path), C.byref(h)))
    return Model(None, h)


RUN_SAVE_IMCIR = 1
CHECK_OVERSHOOT = 1


def run_dir(path: str, device: int = 0, save_imcir: bool = False) -> dict:
    """Render the lines requested by linespectrum.inp in `path`, like the RADlite executable
    (save_imcir: also the circular-image files of a SAVE_IMCIR build)."""
    st = Stats()
    rc = lib().rl_run_dir_ex(os.fsencode(path), device, RUN_SAVE_IMCIR if save_imcir else 0, C.byref(st))
    if rc < 0:
        raise RLError(_err())
    return st.as_dict()


def image_to_spectrum_noalloc(image_ptr: int, nlines: int, nrays: int, nphi: int, nrr: int, nfr: int,
                              ri_ptr: int, scale_ptr: int, flux_ptr: int, precision: int = 0,
                              stream: int = 0, distance_pc: float = 1.0) -> None:
    """rl_image_to_spectrum_noalloc: reduce a device-resident circular image to F_nu.

    For callers that own every device buffer and cannot let the library allocate. All
    pointers are device addresses on the current device. The call only enqueues work on
    `stream` (a cudaStream_t value, 0 = default stream). The ring sums use a fixed 8 MiB
    array inside the library, so calls that overlap on one device race with each other."""
    rc = lib().rl_image_to_spectrum_noalloc(stream or None, precision, image_ptr, nlines, nrays, nphi, nrr, nfr,
                                            ri_ptr, scale_ptr, distance_pc, flux_ptr)
    if rc < 0:
        raise RLError(_err())


def run_manifest(path: str, device: int = 0) -> dict:
    """Render every model directory listed in the manifest file `path` as one batch."""
    st = Stats()
    rc = lib().rl_run_manifest(os.fsencode(path), device, C.byref(st))
    if rc < 0:
        raise RLError(_err())
    return st.as_dict()


def _fnum(txt: str) -> float:
    """A Fortran E/ES field (the 'E' is dropped for three-digit exponents)."""
    t = txt.strip()
    if "E" not in t and "e" not in t:
        for i in range(len(t) - 1, 0, -1):
            if t[i] in "+-" and t[i - 1].isdigit():
                t = t[:i] + "E" + t[i:]
                break
    return float(t)


def read_posvel_file(path: str) -> dict:
    """Parse lineposvel_<mol>_<iline>.dat (the reference's position-velocity layout,
    telescope.F:1965-2016): header fields, velocities [nfr], and the per-channel images of
    3.25465503368e36 I / nu0^2 ("temp") and optical depth ("tau"), each [nfr, ny, nx]."""
    with open(path) as fh:
        L = fh.read().split("\n")
    h = {"version": int(L[1]), "molname": L[2].strip(), "molfile": L[3].strip()}
    h["distance_pc"], h["radvelo"], h["incl_deg"] = _fnum(L[4][0:12]), _fnum(L[4][12:24]), float(L[4][24:31])
    h["up"], h["low"] = int(L[5][0:5]), int(L[5][5:10])
    h["freq"] = _fnum(L[6])
    nfr = h["nfr"] = int(L[7])
    g = L[8]
    nx, ny = int(g[0:5]), int(g[5:10])
    h.update(nx=nx, ny=ny, spx=_fnum(g[10:22]), spy=_fnum(g[22:34]), phioff=float(g[34:41]), xoff=_fnum(g[41:53]),
             yoff=_fnum(g[53:65]))
    i = 10
    h["velo"] = np.array([_fnum(L[i + k]) for k in range(nfr)])
    i += nfr + 1
    temp = np.zeros((nfr, ny, nx))
    tau = np.zeros((nfr, ny, nx))
    for k in range(nfr):
        rows = L[i:i + nx * ny]
        temp[k] = np.array([_fnum(r[0:12]) for r in rows]).reshape(ny, nx)
        tau[k] = np.array([_fnum(r[13:25]) for r in rows]).reshape(ny, nx)
        i += nx * ny + 1
    h["temp"], h["tau"] = temp, tau
    return h


def read_imcir_file(path: str) -> dict:
    """Parse lineposvelcirc_<mol>_<iline>.dat (telescope.F:1346-1373): line frequency, ring
    edges ri [nrr+1] and radii r [nrr+1], and per channel the velocity, the central-beam
    intensity and the [nphi, nrr] intensities and integration mask."""
    with open(path) as fh:
        L = [x for x in fh.read().split("\n")]
    nfr = int(L[0])
    nu0 = _fnum(L[1])
    nphi, nrr = (int(x) for x in L[2].split())
    i = 3
    ri = np.array([_fnum(L[i + k]) for k in range(nrr + 1)]); i += nrr + 1
    rr = np.array([_fnum(L[i + k]) for k in range(nrr + 1)]); i += nrr + 1
    velo, cen = np.zeros(nfr), np.zeros(nfr)
    img = np.zeros((nfr, nphi, nrr))
    mask = np.zeros((nfr, nphi, nrr), dtype=np.uint8)
    for k in range(nfr):
        velo[k] = _fnum(L[i + 1]); cen[k] = _fnum(L[i + 3]); i += 5
        rows = L[i:i + nphi * nrr]
        img[k] = np.array([_fnum(r[0:10]) for r in rows]).reshape(nphi, nrr)
        mask[k] = np.array([int(r[12:13]) for r in rows]).reshape(nphi, nrr)
        i += nphi * nrr
    return {"nfr": nfr, "nu0": nu0, "nphi": nphi, "nrr": nrr, "ri": ri, "r": rr, "velo": velo, "central": cen,
            "image": img, "mask": mask}


def read_spectrum_file(path: str):
    """Parse linespectrum_<mol>.dat (the reference's output layout) into a list of dicts."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    nlines = int(lines[4])
    out, i = [], 6
    for _ in range(nlines):
        up, lo = (int(x) for x in lines[i + 2].split())
        freq = float(lines[i + 3].replace("E", "e") if not lines[i + 3].startswith(".") else "0" + lines[i + 3])
        n = int(lines[i + 5])
        rows = np.array([[float(v) for v in r.split()] for r in lines[i + 7:i + 7 + n]])
        out.append({"up": up, "low": lo, "freq": freq, "velo": rows[:, 0], "flux": rows[:, 1]})
        i += 7 + n - 1
    return out
