"""Ray-sample parity of the circular image (test infrastructure: tests/ and the CPU leg of
bench.py use it as the checker; the product never does).

The oracle renders chosen rays of the circular image of telescope.F:339-631 (its
rlo_line_image, one ray at a time) in a pool of `spawn` processes, one per host core.
The GPU renders the same rays with rl_image_rows. Both are then compared

  * pixel by pixel: |I_gpu - I_oracle| over every sampled ray and channel, relative to the
    brightest sampled pixel of the line (the image's scale), and
  * as a sample spectrum: the image -> F_nu sum of calc_freq_flux_observer
    (telescope.F:1320-1437) over the sampled rays only: the central beam with pi ri(1)^2,
    each ring with pi (ri(j+1)^2 - ri(j)^2) times the mean over its sampled azimuths. The
    reference's spectrum criterion is then applied to it: relative error in every channel
    above 1e-3 of the sample spectrum's peak.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np


def ray_sample(nrays: int, stride: int, offset: int = 0) -> np.ndarray:
    """Rays offset, offset + stride, ... below nrays (ray 0 is the central beam; ray
    1 + (ring-1) nphi + iphi is azimuth iphi of ring `ring`)."""
    return np.arange(offset % stride, nrays, stride, dtype=np.int64)


_ORACLES = {}   # per worker process: loaded models by directory


def _worker(args):
    d, lines, rays = args
    from oracle import pyoracle
    if d not in _ORACLES:
        _ORACLES[d] = pyoracle.Oracle(d)
    o = _ORACLES[d]
    out = np.zeros((len(lines), len(rays), o.nfr))
    counts = np.zeros(3, dtype=np.int64)
    t0 = time.perf_counter()
    for i, il in enumerate(lines):
        for j, r in enumerate(rays):
            img, _, c = o.line_image(int(il), int(r), int(r) + 1)
            out[i, j] = img[0]
            counts += (c["steps"], c["integrated"], c["node_visits"])
    return out, counts, time.perf_counter() - t0


class OraclePool:
    """Host processes (spawn) that render oracle image rows; each keeps the models it has
    loaded, so repeated calls on one directory pay the parse once."""

    def __init__(self, procs: int | None = None):
        self.procs = procs or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.procs)

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def rows(self, d: str, lines, rays):
        """Oracle image rows [len(lines), len(rays), nfr] of model directory d (rays dealt
        round-robin over the processes). Returns (rows, counts, compute_s, wall_s): counts =
        (steps, integrated, node visits) summed, compute_s = the busiest process's compute
        time (model loading excluded), wall_s = the call's wall time."""
        rays = np.asarray(rays)
        lines = list(lines)
        idx = [np.arange(i, len(rays), self.procs) for i in range(self.procs)]
        idx = [ix for ix in idx if len(ix)]
        t0 = time.perf_counter()
        res = self.pool.map(_worker, [(d, lines, rays[ix]) for ix in idx], chunksize=1)
        wall = time.perf_counter() - t0
        return _gather(res, idx, len(lines), len(rays)) + (wall,)


def oracle_rows(d: str, lines, rays, procs: int | None = None):
    """OraclePool.rows on a pool of its own."""
    with OraclePool(procs) as pool:
        return pool.rows(d, lines, rays)


def _gather(res, idx, nl, nsel):
    nfr = res[0][0].shape[2]
    rows = np.zeros((nl, nsel, nfr))
    counts = np.zeros(3, dtype=np.int64)
    for ix, (r, c, _) in zip(idx, res):
        rows[:, ix] = r
        counts += c
    return rows, counts, max(r[2] for r in res)


def sample_spectrum(rows: np.ndarray, rays, ri: np.ndarray, nphi: int) -> np.ndarray:
    """F_nu sum (up to the common factor 1/d^2) over the sampled rays: rows [..., nsel, nfr]
    -> [..., nfr]. Rings without a sampled ray drop out; the central beam counts when
    sampled."""
    rays = np.asarray(rays)
    out = np.zeros(rows.shape[:-2] + rows.shape[-1:])
    pi = 3.14159265359
    central = np.flatnonzero(rays == 0)
    if len(central):
        out += pi * ri[1] ** 2 * rows[..., central[0], :]
    ring = (rays[rays > 0] - 1) // nphi + 1
    sel = np.flatnonzero(rays > 0)
    for j in np.unique(ring):
        m = sel[ring == j]
        out += pi * (ri[j + 1] ** 2 - ri[j] ** 2) * rows[..., m, :].mean(axis=-2)
    return out


def spectrum_relerr(got: np.ndarray, ref: np.ndarray) -> float:
    """Largest relative error over the channels above 1e-3 of the reference's peak."""
    sel = ref > 1e-3 * ref.max()
    if not sel.any():
        return 0.0
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


def pixel_relerr(got: np.ndarray, ref: np.ndarray) -> float:
    """Largest |got - ref| over the pixels of one line's sample ([nsel, nfr]) relative to the
    brightest oracle pixel of that sample."""
    scale = float(np.abs(ref).max())
    diff = float(np.abs(got - ref).max())
    if scale == 0.0:
        return 0.0 if diff == 0.0 else float("inf")
    return diff / scale


def compare(gpu_rows: np.ndarray, ora_rows: np.ndarray, rays, ri: np.ndarray, nphi: int) -> dict:
    """Per-line errors of a ray sample ([nlines, nsel, nfr] each): the sample-spectrum
    criterion, the pixel error, and the number of channels the criterion checked."""
    gs = sample_spectrum(gpu_rows, rays, ri, nphi)
    os_ = sample_spectrum(ora_rows, rays, ri, nphi)
    spec = [spectrum_relerr(gs[i], os_[i]) for i in range(gs.shape[0])]
    pix = [pixel_relerr(gpu_rows[i], ora_rows[i]) for i in range(gs.shape[0])]
    checked = [int(np.count_nonzero(os_[i] > 1e-3 * os_[i].max())) for i in range(gs.shape[0])]
    return {"spectrum_rel_err": spec, "pixel_rel_err": pix, "channels_checked": checked}


def render_params(args):
    """Oracle spectra of the named synthetic model with per-cell parameters (ln T, ln X,
    width; the differentiable path's cell order) written in the reference's formats to a
    fresh directory: (flux [nlines, nfr] of the model's lines, steps, integrated)."""
    import shutil
    import tempfile
    from oracle import pyoracle
    from radlite_gb300 import synth
    name, lnT, lnX, width = args
    cfg = synth.config_by_name(name)
    d = tempfile.mkdtemp(prefix="fd_")
    try:
        synth.write_model(cfg, d, fields=synth.lte_fields(cfg, lnT, lnX, width))
        o = pyoracle.Oracle(d)
        out, steps, integ = [], 0, 0
        for k in range(cfg.nlines):
            f, _, cnt = o.line_spectrum(cfg.ilinestart + k)
            out.append(f)
            steps += cnt["steps"]
            integ += cnt["integrated"]
        return np.array(out), steps, integ
    finally:
        shutil.rmtree(d, ignore_errors=True)
