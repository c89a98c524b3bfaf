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
        L.rlo_ray_spectrum.argtypes = [vp, C.c_int, C.c_double, C.c_double, _D, _D]
        L.rlo_line_image.argtypes = [vp, C.c_int, C.c_int, C.c_int, _D, C.POINTER(C.c_ubyte), C.POINTER(C.c_longlong)]
        L.rlo_image_to_spectrum.argtypes = [vp, _D, _D]
        L.rlo_line_spectrum.argtypes = [vp, C.c_int, _D, _D, C.POINTER(C.c_longlong)]
        L.rlo_pv_request.argtypes = [vp, _I, _D]
        L.rlo_pv_rays.argtypes = [vp, C.c_int, C.c_int] + [C.c_double] * 5 + [C.c_int, _D, _D, _D, _I, _D]
        L.rlo_posvel.argtypes = [vp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 5 + [C.c_int, _D, _D]
        L.rlo_run_dir.argtypes = [C.c_char_p]
        L.rlo_masing.argtypes = [vp]
        L.rlo_overshoots.argtypes = [vp]
        L.rlo_overshoots.restype = C.c_longlong
        L.rlo_hunt.argtypes = [_D, C.c_int, C.c_double, C.c_int]
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
        pi = np.zeros(4, dtype=np.int32)
        pd = np.zeros(5)
        lib().rlo_pv_request(self.h, pi.ctypes.data_as(_I), _dp(pd))
        self.command = int(pi[0])
        self.pv = dict(nx=int(pi[1]), ny=int(pi[2]), szimx=float(pd[0]), szimy=float(pd[1]), phioff=float(pd[2]),
                       xoff=float(pd[3]), yoff=float(pd[4]), addstar=int(pi[3]))

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

    def ray_spectrum(self, iline: int, x0: float, z0: float):
        """I and the line-of-sight optical depth of every channel along one ray (x0, z0):
        one pixel of the rectangular (position-velocity) image."""
        I, tau = np.zeros(self.nfr), np.zeros(self.nfr)
        rc = lib().rlo_ray_spectrum(self.h, iline, float(x0), float(z0), _dp(I), _dp(tau))
        if rc != 0:
            raise OracleError(lib().rlo_last_error().decode())
        return I, tau

    def pv_rays(self, nx, ny, szimx, szimy, phioff=0.0, xoff=0.0, yoff=0.0, addstar=0):
        """Pixel rays of the rectangular camera: x0, z0, b [nx*ny] (ix outer, iy inner) and
        (starunres, spx, spy, srat, theta0)."""
        n = nx * ny
        x0, z0, b = np.zeros(n), np.zeros(n), np.zeros(n)
        iv = np.zeros(1, dtype=np.int32)
        dv = np.zeros(4)
        rc = lib().rlo_pv_rays(self.h, nx, ny, szimx, szimy, phioff, xoff, yoff, addstar, _dp(x0), _dp(z0), _dp(b),
                               iv.ctypes.data_as(_I), _dp(dv))
        if rc != 0:
            raise OracleError(lib().rlo_last_error().decode())
        return x0, z0, b, (int(iv[0]), *(float(v) for v in dv))

    def posvel(self, iline, nx, ny, szimx, szimy, phioff=0.0, xoff=0.0, yoff=0.0, addstar=0):
        """Intensity and optical-depth cube [nfr, ny, nx] of one line."""
        I = np.zeros((self.nfr, ny, nx))
        tau = np.zeros((self.nfr, ny, nx))
        rc = lib().rlo_posvel(self.h, iline, nx, ny, szimx, szimy, phioff, xoff, yoff, addstar, _dp(I), _dp(tau))
        if rc != 0:
            raise OracleError(lib().rlo_last_error().decode())
        return I, tau

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

    def masing(self) -> bool:
        """Whether the last line spectrum, image or cube met the masing test."""
        return bool(lib().rlo_masing(self.h))

    def overshoots(self) -> int:
        """Formal-solution steps of the last line spectrum, image or cube whose quadrature
        exceeded twice the theoretical maximum before the bracket."""
        return int(lib().rlo_overshoots(self.h))


def run_dir(path: str) -> None:
    if lib().rlo_run_dir(os.fsencode(path)) != 0:
        raise OracleError(lib().rlo_last_error().decode())
