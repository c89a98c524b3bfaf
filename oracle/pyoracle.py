"""ctypes access to the CPU oracle (test infrastructure: tests/, smoke() and the CPU
baseline of bench.py use it as the checker; the product never does)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librloracle.so")
EXE = os.path.join(BUILD, "rl_oracle")
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.rlo_last_error.restype = C.c_char_p
        L.rlo_load_dir.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.rlo_free.argtypes = [vp]
        L.rlo_info.argtypes = [vp, _I, _D]
        L.rlo_rays.argtypes = [vp, _D, _D, _D, _D]
        L.rlo_trajectory.argtypes = [vp, C.c_int, C.c_int, _D, _D, _D, _D, _D, _I, _I, _I]
        L.rlo_line_image.argtypes = [vp, C.c_int, C.c_int, C.c_int, _D, C.POINTER(C.c_ubyte), C.POINTER(C.c_longlong)]
        L.rlo_image_to_spectrum.argtypes = [vp, _D, _D]
        L.rlo_line_spectrum.argtypes = [vp, C.c_int, _D, _D, C.POINTER(C.c_longlong)]
        L.rlo_run_dir.argtypes = [C.c_char_p]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _dp(a):
    return a.ctypes.data_as(_D)


class Oracle:
    def __init__(self, path: str):
        self.h = C.c_void_p()
        if lib().rlo_load_dir(os.fsencode(path), C.byref(self.h)) != 0:
            raise OracleError(lib().rlo_last_error().decode())
        iv = np.zeros(10, dtype=np.int32)
        dv = np.zeros(5)
        lib().rlo_info(self.h, iv.ctypes.data_as(_I), _dp(dv))
        (self.nr, self.nth, self.nlines_spec, self.ilinestart, self.nfr, self.nrays, self.nphi, self.nrr,
         self.nlines_mol, self.nlev) = (int(x) for x in iv)
        self.incl_rad, self.vmax, self.rstar, self.aksmax, self.theta0 = (float(x) for x in dv)

    def __del__(self):
        if getattr(self, "h", None):
            lib().rlo_free(self.h)
            self.h = None

    def rays(self):
        x0, z0 = np.zeros(self.nrays), np.zeros(self.nrays)
        rr, ri = np.zeros(self.nrr + 1), np.zeros(self.nrr + 2)
        lib().rlo_rays(self.h, _dp(x0), _dp(z0), _dp(rr), _dp(ri))
        return x0, z0, rr, ri

    def trajectory(self, iray: int, cap: int = 8192) -> dict:
        d = {k: np.zeros(cap) for k in ("s", "r", "theta", "mu", "phi")}
        i = {k: np.zeros(cap, dtype=np.int32) for k in ("icr", "ir", "it")}
        n = lib().rlo_trajectory(self.h, iray, cap, *(_dp(d[k]) for k in ("s", "r", "theta", "mu", "phi")),
                                 *(i[k].ctypes.data_as(_I) for k in ("icr", "ir", "it")))
        if n < 0:
            raise OracleError(lib().rlo_last_error().decode())
        out = {k: v[:n] for k, v in d.items()}
        out.update({k: v[:n] for k, v in i.items()})
        return out

    def line_image(self, iline: int, ray_begin: int = 0, ray_end: int | None = None):
        ray_end = self.nrays if ray_end is None else ray_end
        n = ray_end - ray_begin
        img = np.zeros((n, self.nfr))
        mask = np.zeros((n, self.nfr), dtype=np.uint8)
        cnt = np.zeros(3, dtype=np.int64)
        rc = lib().rlo_line_image(self.h, iline, ray_begin, ray_end, _dp(img),
                                  mask.ctypes.data_as(C.POINTER(C.c_ubyte)), cnt.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc != 0:
            raise OracleError(lib().rlo_last_error().decode())
        return img, mask, {"steps": int(cnt[0]), "integrated": int(cnt[1]), "node_visits": int(cnt[2])}

    def image_to_spectrum(self, img):
        flux = np.zeros(self.nfr)
        lib().rlo_image_to_spectrum(self.h, _dp(np.ascontiguousarray(img)), _dp(flux))
        return flux

    def line_spectrum(self, iline: int):
        flux, velo = np.zeros(self.nfr), np.zeros(self.nfr)
        cnt = np.zeros(3, dtype=np.int64)
        rc = lib().rlo_line_spectrum(self.h, iline, _dp(flux), _dp(velo), cnt.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc != 0:
            raise OracleError(lib().rlo_last_error().decode())
        return flux, velo, {"steps": int(cnt[0]), "integrated": int(cnt[1]), "node_visits": int(cnt[2])}


def run_dir(path: str) -> None:
    if lib().rlo_run_dir(os.fsencode(path)) != 0:
        raise OracleError(lib().rlo_last_error().decode())
