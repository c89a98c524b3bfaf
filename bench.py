"""Benchmark of the GB300 line raytrace on the large band workload.

Workload (one step): the 400x200 (r, theta) disk with seeded +-10% lognormal per-cell
perturbations of T and rho, 20 ro-vibrational lines (P and R branch, J=1..10) x 200
channels (+-24.875 km/s), circular image of 1000 rings x 256 azimuths (+1 central beam),
inclinations 20 and 60 degrees: 40 spectra, 2.048e9 ray-channels. Synthetic inputs
(radlite_gb300.synth); FP64 geometry, FP32 transfer.

  value   ray-channels/s with the model resident on the device, timed with CUDA events on
          the library's stream (geometry + walk + reduction of both inclinations)
  e2e     the same metric through the C ABI from host arrays: model upload, both
          inclinations and the spectra read back, wall clock
  --impl reference   the reference algorithm on the host cores: the FP64 C restatement of
          RADLite's Fortran raytrace (the Fortran itself does not compile here), one
          process per core, on a bounded sample of the same workload.

The same JSON line carries the other halves of the metric (plain vs batched+adjoint):
  batched  256 uneven models rendered by one graph-replayed launch sequence against the
           same models one per-model call at a time (spectra/s of each, same spectra)
  adjoint  forward and adjoint times of the differentiable raytrace on the 200x100 disk
           (10 lines x 128 channels, 600x128 rays; per-cell ln T, ln X, width gradients)
  fit      the batched forward+adjoint fitting step on 64 uneven models (20 lines x 200
           channels, 4 disk-law parameters each) against plain per-model forward + central
           finite differences (9 forwards per gradient)
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ray-channels/s & spectra/s at 1e-4 rel err: plain vs batched+adjoint, 1 GB300"
UNIT = "ray-channels/s"
INCLS = (20.0, 60.0)
# per formal-solution step: minimal FP32-pipe instructions and MUFU operations of the
# linear-source step with a Gaussian profile (Doppler offset, profile, emissivity and
# extinction, optical depth, exponential coefficients, bracket, intensity update)
BUDGET_FP32 = 19
BUDGET_MUFU = 3
CONFIG = {"workload": "band_large: 400x200 disk (+-10% lognormal T, rho), 20 band lines x 200 channels, "
                      "1000x256+1 rays, incl 20+60 deg",
          "l2": "inputs larger than L2 (node records ~10 GB per inclination)"}


def workload():
    from radlite_gb300 import synth
    cfg = synth.config_by_name("band_large")
    return cfg, synth.model_arrays(cfg)


def camera(cfg, incl):
    return dict(incl_deg=incl, nphi=cfg.nphi, dbdr=cfg.dbdr, nrrayextra=cfg.nrrextra, vmax=cfg.vmax, dv=cfg.dv,
                ilinestart=cfg.ilinestart, nlines=cfg.nlines)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.rows, self.proc = device, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 4 + i and r[4 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------
# CPU side: the oracle on a bounded ray sample (one process per core), also the checker
# ------------------------------------------------------------------------------------
def model_dirs(tmp):
    """The band workload written in the reference's file formats, one directory per
    inclination (the oracle's input, and the GPU model's for the timing and the parity)."""
    from radlite_gb300 import synth
    dirs = {}
    for inc in INCLS:
        d = os.path.join(tmp, f"band_large_i{inc:.0f}")
        if not os.path.exists(os.path.join(d, "radlite.inp")):
            synth.write_model(synth.config_by_name("band_large", incl_deg=inc), d)
        dirs[inc] = d
    return dirs


def n_rays(cfg):
    return 1 + (abs(cfg.nrrextra) + 10 + cfg.dbdr * (cfg.nr - 1)) * cfg.nphi


def oracle_sample(pool, dirs, cfg, stride, offset=0):
    """The oracle's image rows of every stride-th ray (from `offset`) of every line at every
    inclination: the ray-channels/s of that sample on the pool's host processes, and the
    rows themselves (per inclination, [nlines, nsel, nfr])."""
    from oracle import sample
    rays = sample.ray_sample(n_rays(cfg), stride, offset)
    lines = range(cfg.ilinestart, cfg.ilinestart + cfg.nlines)
    nfr = int(2.0 * cfg.vmax / cfg.dv + 1)
    rows, compute = {}, 0.0
    for inc, d in dirs.items():
        r, _, comp, _ = pool.rows(d, lines, rays)
        rows[inc] = r
        compute += comp
    n = len(rays) * nfr * cfg.nlines * len(dirs)
    return rays, rows, {"ray_channels": n, "rays": len(rays), "compute_s": compute, "value": n / compute}


def sample_text(cfg, stride, nsel, offset=0):
    first = f" from ray {offset % stride}" if offset % stride else ""
    return (f"every {stride}th ray{first} ({nsel} rays x {int(2.0 * cfg.vmax / cfg.dv + 1)} channels) of all "
            f"{cfg.nlines} lines at both inclinations ({'+'.join(f'{i:.0f}' for i in INCLS)} deg)")


def cpu_model() -> str:
    """The host CPU as lscpu names it (architecture and model)."""
    import platform
    name = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return f"{platform.machine()} {name}".strip()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def max_over_ranks(x: float, dist) -> float:
    """The largest of every rank's `x` (the job's time is its slowest replica's); `x`
    itself with one rank. Replicas exchange nothing else."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_arm(args):
    world, rank, _, dist = dist_setup()
    if rank != 0:
        return 0
    from oracle import sample
    cfg, _ = workload()
    procs = os.cpu_count() or 1
    stride = args.ref_stride
    with tempfile.TemporaryDirectory() as tmp, sample.OraclePool(procs) as pool:
        dirs = model_dirs(tmp)
        vals = []
        for i in range(args.warmup + args.steps):
            _, _, st = oracle_sample(pool, dirs, cfg, stride, offset=i)
            if i >= args.warmup:
                vals.append(st)
    v = statistics.median(x["value"] for x in vals)
    ms = statistics.median(x["compute_s"] for x in vals) * 1e3
    smp = (sample_text(cfg, stride, vals[0]["rays"]) + "; step i starts at ray i, so successive steps render "
           "different rays")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator in the reference file formats)",
            "config": CONFIG,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "cpu": cpu_model(), "kind": "port",
                             "sample": smp},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference Fortran cannot be compiled on this image (no Fortran compiler); timed is the "
                    "FP64 C restatement of its raytrace (oracle/), one process per host core"}
    print(json.dumps(line), flush=True)
    return 0


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def load_measured():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def parity_case(ctx, dirs, cfg, rays, ora, stride):
    """GPU image rows of the oracle's ray sample (same model directories, same rays, FP32
    transfer) against the oracle's: per spectrum (line, inclination) the sample-spectrum
    error in every channel above 1e-3 of its peak and the pixel error (oracle/sample.py)."""
    from oracle import pyoracle, sample
    per_spec, per_pix, checked, names = [], [], [], []
    for inc, d in dirs.items():
        _, _, _, ri = pyoracle.Oracle(d).rays()
        m = ctx.load_dir(d)
        _, rows = m.image_rows(cfg.ilinestart, cfg.nlines, rays)
        m.free()
        c = sample.compare(rows, ora[inc], rays, ri, cfg.nphi)
        per_spec += c["spectrum_rel_err"]
        per_pix += c["pixel_rel_err"]
        checked += c["channels_checked"]
        names += [f"line {cfg.ilinestart + k} incl {inc:.0f}" for k in range(cfg.nlines)]
    return {"criterion": "relative error in every channel above 1e-3 of the peak <= 1e-4 (sample spectrum: the "
                         "image->F_nu sum over the sampled rays), GPU FP32 transfer vs FP64 oracle",
            "sample": sample_text(cfg, stride, len(rays)), "spectra": len(per_spec), "spectrum_names": names,
            "max_spectrum_rel_err": max(per_spec), "per_spectrum_rel_err": per_spec,
            "max_pixel_rel_err": max(per_pix), "per_spectrum_pixel_rel_err": per_pix,
            "channels_checked": checked, "channels_checked_total": int(sum(checked)),
            "pass": bool(max(per_spec) <= 1e-4)}


def disk_line_case(ctx, pool, tmp, steps):
    """The plain single-model configuration: the 100x60 disk, line J=3-2 x 64 channels,
    400 rings x 128 azimuths + the central beam, incl 45 deg. Device and end-to-end
    ray-channels/s, and the full spectrum against the oracle's (all 51,201 rays rendered by
    the host pool and summed by the oracle), FP32 and FP64 transfer."""
    import numpy as np
    from radlite_gb300 import synth
    from oracle import pyoracle, sample
    cfg = synth.config_by_name("disk_line")
    d = os.path.join(tmp, "disk_line")
    synth.write_model(cfg, d)
    il = cfg.ilinestart
    m = ctx.load_dir(d)
    for _ in range(3):
        m.set_camera(cfg.incl_deg, cfg.nphi, cfg.dbdr, cfg.nrrextra)
        m.spectra(il, 1)
    dev = []
    for _ in range(max(1, steps)):
        m.set_camera(cfg.incl_deg, cfg.nphi, cfg.dbdr, cfg.nrrextra)
        f32, st = m.spectra(il, 1, stats=True)
        dev.append(st["geometry_ms"] + st["upload_ms"] + st["walk_ms"] + st["reduce_ms"])
    rc = st["ray_channels"]
    arr = synth.model_arrays(cfg)
    e2e = []
    for _ in range(3):
        t0 = time.perf_counter()
        m2 = ctx.load_arrays(arr, camera(cfg, cfg.incl_deg))
        m2.spectra(il, 1)
        e2e.append(time.perf_counter() - t0)
        m2.free()
    o = pyoracle.Oracle(d)
    rows, counts, comp, _ = pool.rows(d, [il], np.arange(o.nrays))
    ref = o.image_to_spectrum(rows[0])
    m.set_precision(1)
    f64, st64 = m.spectra(il, 1, stats=True)
    m.free()
    ms = statistics.median(dev)
    return {"workload": f"disk_line: {cfg.nr}x{cfg.nt} disk, line {il} (J=3-2) x {st['nfr']} channels, "
                        f"{st['nrays']} rays, incl {cfg.incl_deg:.0f} deg",
            "ms_per_step": ms, "value": rc / (ms * 1e-3), "unit": UNIT, "spectra_per_s": 1.0 / (ms * 1e-3),
            "e2e": {"value": rc / statistics.median(e2e), "unit": UNIT},
            "parity": {"fp32_rel_err": sample.spectrum_relerr(f32[0], ref),
                       "fp64_rel_err": sample.spectrum_relerr(f64[0], ref),
                       "fp64_integrated_equal": bool(st64["integrated"] == counts[1]),
                       "fp64_steps": int(st64["steps"]), "oracle_steps": int(counts[0]),
                       "criterion": "full spectrum, every channel above 1e-3 of the peak"},
            "cpu_baseline": {"value": rc / comp, "unit": UNIT, "cores": pool.procs, "kind": "port",
                             "sample": "every ray and channel (the whole configuration)"}}


def ours(args):
    import numpy as np
    import radlite_gb300 as rl
    from oracle import sample
    world, rank, local, dist = dist_setup()
    cfg, arr = workload()
    tmpd = tempfile.TemporaryDirectory()
    dirs = model_dirs(tmpd.name)
    # the checker's host processes (spawn) start before the first CUDA call
    pool = sample.OraclePool() if rank == 0 and not args.no_cpu else None
    ctx = rl.Context(local)
    peaks = ctx.measure_peaks()
    m = ctx.load_dir(dirs[INCLS[0]])

    def step(model):
        st_all = []
        spectra = []
        for inc in INCLS:
            model.set_camera(inc, cfg.nphi, cfg.dbdr, cfg.nrrextra)
            f, st = model.spectra(cfg.ilinestart, cfg.nlines, stats=True)
            spectra.append(f)
            st_all.append(st)
        return spectra, st_all

    for _ in range(args.warmup):
        step(m)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    dev_ms, walk_ms, steps_fs, integ = [], [], 0, 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            _, sts = step(m)
            dev_ms.append(sum(s["geometry_ms"] + s["upload_ms"] + s["walk_ms"] + s["reduce_ms"] for s in sts))
            walk_ms.append(sum(s["walk_ms"] for s in sts))
            steps_fs = sum(s["steps"] for s in sts)
            integ = sum(s["integrated"] for s in sts)
            passes = sum(s["node_passes"] for s in sts)
            packed = sum(s["packed_passes"] for s in sts)
            empty = sum(s["empty_steps"] for s in sts)
            refined = sum(s["refined_passes"] for s in sts)
            substeps = sum(s["sub_steps"] for s in sts)
    wall = (time.perf_counter() - t0) / args.steps
    ms = max_over_ranks(sum(dev_ms) / len(dev_ms), dist)
    nrays = n_rays(cfg)
    nfr = int(2.0 * cfg.vmax / cfg.dv + 1)
    rc_per_step = nrays * nfr * cfg.nlines * len(INCLS)
    value = world * rc_per_step / (ms * 1e-3)
    spectra_s = world * cfg.nlines * len(INCLS) / (ms * 1e-3)
    # roofline of the walk kernel (dominant): FP32 / MUFU issue with the per-step budget
    wk = sum(walk_ms) / len(walk_ms) * 1e-3
    # steps of empty segments (zero emissivity and opacity at both ends) are counted by the
    # reference but take no arithmetic here: the roofline counts the executed steps
    executed = steps_fs - empty
    t_fp = executed * BUDGET_FP32 / peaks["ffma_per_s"]
    t_mu = executed * BUDGET_MUFU / peaks["ex2_per_s"]
    bound_mufu = t_mu >= t_fp
    achieved = (executed * (BUDGET_MUFU if bound_mufu else BUDGET_FP32)) / wk
    peak = peaks["ex2_per_s"] if bound_mufu else peaks["ffma_per_s"]
    traffic = load_traffic().get("k_walk_dram_bytes_per_launch")
    hbm_peak = load_measured().get("hbm_gbs")
    traffic_gbs = traffic / (wk / len(INCLS)) / 1e9 if traffic else None
    # e2e: through the C ABI from host arrays, wall clock, copies included
    e2e_t, h2d, d2h = [], 0, 0
    for i in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        m2 = ctx.load_arrays(arr, camera(cfg, INCLS[0]))
        spectra, sts = step(m2)
        e2e_t.append(time.perf_counter() - t1)
        h2d = sum(s["h2d_bytes"] for s in sts)
        d2h = sum(s["d2h_bytes"] for s in sts)
        m2.free()
    e2e = world * rc_per_step / max_over_ranks(statistics.median(e2e_t), dist)
    # accuracy at full size: FP32 vs FP64 of the first line at the first inclination
    rel = None
    if not args.no_verify:
        m.set_camera(INCLS[0], cfg.nphi, cfg.dbdr, cfg.nrrextra)
        f32 = m.spectra(cfg.ilinestart, 1)[0]
        m.set_precision(1)
        f64 = m.spectra(cfg.ilinestart, 1)[0]
        m.set_precision(0)
        sel = f64 > 1e-3 * f64.max()
        rel = float(np.max(np.abs(f32[sel] - f64[sel]) / np.abs(f64[sel])))
    m.free()
    batched = adjoint = fitting = None
    if rank == 0 and args.batch_models > 0:
        batched = batched_case(ctx, args.batch_models, 2)
    if rank == 0 and not args.no_diff:
        adjoint = adjoint_case(ctx)
        fitting = fit_case(ctx, args.fit_models, args.fit_steps, nphi=args.fit_nphi, dbdr=args.fit_dbdr)
        if args.recovery_steps > 0:
            fitting["recovery"] = recovery_case(ctx, steps=args.recovery_steps)
    out = None
    if rank == 0:
        cpu = parity = disk = None
        extras = {}
        if pool is not None:
            rays, ora, s = oracle_sample(pool, dirs, cfg, args.cpu_stride)
            cpu = {"value": s["value"], "unit": UNIT, "cores": pool.procs, "cpu": cpu_model(), "kind": "port",
                   "sample": sample_text(cfg, args.cpu_stride, s["rays"]) + ", FP64 C restatement, one process per core"}
            parity = parity_case(ctx, dirs, cfg, rays, ora, args.cpu_stride)
            del ora
            disk = disk_line_case(ctx, pool, tmpd.name, args.steps)
        if not args.no_extras:
            extras = extras_case(ctx, cfg, arr, dirs[INCLS[0]], tmpd.name, with_cpu=not args.no_cpu)
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "wall_ms_per_step": wall * 1e3,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (fp64 geometry)",
               "data": "synthetic (seeded generator in the reference file formats)",
               "config": CONFIG, "ray_channels_per_step": rc_per_step, "spectra_per_step": cfg.nlines * len(INCLS),
               "spectra_per_s": spectra_s,
               "formal_solution_steps_per_step": steps_fs, "integrated_ray_channels_per_step": integ,
               "rel_err_fp32_vs_fp64": rel,
               "parity": parity,
               "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "path": "rl_load_arrays from host arrays + rl_spectra per inclination, wall clock"},
               "roofline": {"bound": "mufu_issue" if bound_mufu else "fp32_issue", "achieved": achieved / 1e12,
                            "peak": peak / 1e12, "unit": "Tops/s", "frac": achieved / peak, "traffic": traffic,
                            "kernel": "k_walk<float>", "walk_ms_per_step": wk * 1e3,
                            "executed_steps_per_step": executed, "empty_steps_per_step": empty,
                            "node_passes_per_step": passes, "packed_fraction": packed / passes if passes else None,
                            "refined_fraction": refined / passes if passes else None,
                            "sub_steps_per_step": substeps,
                            "budget_per_step": {"fp32": BUDGET_FP32, "mufu": BUDGET_MUFU},
                            "peaks_measured": peaks,
                            "hbm_side": {"traffic_gb_per_s": traffic_gbs, "peak_gb_per_s": hbm_peak,
                                         "frac_of_measured": (traffic_gbs / hbm_peak
                                                              if traffic_gbs and hbm_peak else None)}},
               "disk_line": disk,
               "batched": batched,
               "adjoint": adjoint,
               "fit": fitting,
               "posvel": extras.get("posvel"),
               "genspec": extras.get("genspec"),
               "input": extras.get("input"),
               "cpu_baseline": cpu,
               "clocks": clk.summary(),
               "gpu_launches": args.steps * len(INCLS) * 4}
        print(json.dumps(out), flush=True)
    if pool is not None:
        pool.close()
    ctx.close()
    tmpd.cleanup()
    return 0


def extras_case(ctx, cfg, arr, d, tmp, with_cpu=True):
    """The rows beside the raytrace: the position-velocity cube of the band_large disk, the
    spectrum post-processing of a 2000-line band, and the input parsing of the band_large
    directory (text and binary cache). Each with its CPU counterpart where it has one."""
    import numpy as np
    import radlite_gb300 as rl
    from radlite_gb300 import synth
    out = {}
    # position-velocity cube: 256 x 256 pixels over the disk diameter, 4 lines x 200 channels
    m = ctx.load_arrays(arr, camera(cfg, INCLS[0]))
    size = 2.0 * float(arr["r"][-1])
    npx, nl = 256, 4
    m.set_posvel(npx, npx, size, size, addstar=1)
    m.posvel(cfg.ilinestart, nl)
    runs = []
    for _ in range(3):
        t0 = time.perf_counter()
        _, _, st = m.posvel(cfg.ilinestart, nl, stats=True)
        runs.append((time.perf_counter() - t0, st))
    wall = statistics.median(r[0] for r in runs)
    st = runs[-1][1]
    dev_ms = st["geometry_ms"] + st["upload_ms"] + st["walk_ms"] + st["reduce_ms"]
    pv = {"workload": f"band_large incl {INCLS[0]:.0f} deg, {npx}x{npx} pixels over the disk diameter, "
                      f"lines {cfg.ilinestart}-{cfg.ilinestart + nl - 1} x 200 channels, intensity and optical depth",
          "traced_rays": st["nrays"], "ray_channels": st["ray_channels"], "device_ms": dev_ms, "walk_ms": st["walk_ms"],
          "geometry_ms": st["geometry_ms"], "ray_channels_per_s": st["ray_channels"] / (dev_ms * 1e-3),
          "e2e_ray_channels_per_s": st["ray_channels"] / wall, "d2h_bytes": st["d2h_bytes"]}
    m.free()
    if with_cpu:
        from oracle import pyoracle
        o = pyoracle.Oracle(d)
        x0, z0, b, _ = o.pv_rays(npx, npx, size, size, 0.0, 0.0, 0.0, 1)
        inside = np.flatnonzero(b < 0.999 * float(arr["r"][-1]))
        pick = inside[:: max(1, len(inside) // 16)][:16]
        t0 = time.perf_counter()
        for r in pick:
            o.ray_spectrum(cfg.ilinestart, x0[r], z0[r])
        cpu_s = time.perf_counter() - t0
        pv["cpu_baseline"] = {"value": len(pick) * o.nfr / cpu_s, "unit": "ray-channels/s", "cores": 1, "kind": "port",
                              "sample": f"{len(pick)} pixel rays x {o.nfr} channels of line {cfg.ilinestart}, FP64 C "
                                        "restatement, one core"}
        del o
    out["posvel"] = pv
    # spectrum post-processing of a 2000-line band (201 channels per line)
    rng = np.random.default_rng(5)
    lines = []
    vel = np.linspace(-20.0, 20.0, 201)
    for i in range(2000):
        flux = (1 + 0.001 * vel) * rng.uniform(1e-20, 2e-20) + rng.uniform(0, 4e-20) * np.exp(-(vel / rng.uniform(2, 6)) ** 2)
        lines.append({"vel": vel, "flux": flux, "freq": 2.99792458e10 * rng.uniform(2000.0, 2200.0), "maxnumpoints": 201})
    ctx.gen_spec(lines, 3.0, 1.0, 140.0)
    gs = []
    for _ in range(3):
        t0 = time.perf_counter()
        o2 = ctx.gen_spec(lines, 3.0, 1.0, 140.0, stats=True)
        gs.append((time.perf_counter() - t0, o2["stats"]))
    g = {"workload": "2000 lines x 201 channels over 2000-2200 cm^-1, obsres 3 km/s, sampling 1 km/s",
         "fine_points": gs[-1][1]["nrays"], "output_points": gs[-1][1]["nfr"],
         "device_ms": gs[-1][1]["upload_ms"] + gs[-1][1]["walk_ms"], "e2e_ms": statistics.median(x[0] for x in gs) * 1e3}
    if with_cpu:
        from oracle import genspec_ref
        t0 = time.perf_counter()
        ref = genspec_ref.process(lines, 3.0, 1.0, 140.0)
        g["cpu_baseline"] = {"value": (time.perf_counter() - t0) * 1e3, "unit": "ms", "cores": 1, "kind": "port",
                             "sample": "the whole workload, numpy restatement of _process_spectrum"}
        g["max_rel_diff_vs_cpu"] = float(np.max(np.abs(o2["spectrum"] - ref["spectrum"]) / np.abs(ref["spectrum"]).max()))
    out["genspec"] = g
    # input parsing of the band_large directory: text, then the binary cache
    t0 = time.perf_counter()
    rl.load_dir_host(d).free()
    text_s = time.perf_counter() - t0
    cache = os.path.join(tmp, "input_cache")
    os.makedirs(cache, exist_ok=True)
    old = os.environ.get("RLGPU_INPUT_CACHE")
    os.environ["RLGPU_INPUT_CACHE"] = cache
    rl.load_dir_host(d).free()
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        rl.load_dir_host(d).free()
        ts.append(time.perf_counter() - t0)
    if old is None:
        del os.environ["RLGPU_INPUT_CACHE"]
    else:
        os.environ["RLGPU_INPUT_CACHE"] = old
    nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
    out["input"] = {"workload": f"band_large input directory ({nbytes / 1e6:.0f} MB of text)",
                    "text_parse_s": text_s, "cached_load_s": statistics.median(ts)}
    return out


def batched_case(ctx, n_models, steps, tune_stride=8):
    """Plain per-model launches against one batched, graph-replayed launch sequence on the
    uneven multi-model workload (synth.batch_configs): same spectra, spectra/s of each."""
    import numpy as np
    import radlite_gb300 as rl
    from radlite_gb300 import synth
    cfgs = synth.batch_configs(n_models)
    cams = [camera(c, c.incl_deg) for c in cfgs]
    nspec = sum(c.nlines for c in cfgs)
    # plain: one model at a time, as a driver loop over model directories would run it
    plain, t_cold, t_warm, rc_total = [], 0.0, 0.0, 0
    for c, cam in zip(cfgs, cams):
        m = ctx.load_arrays(synth.model_arrays(c), cam)
        t0 = time.perf_counter()
        m.spectra(c.ilinestart, c.nlines)                    # geometry, line tables, walk, reduction
        t1 = time.perf_counter()
        f, st = m.spectra(c.ilinestart, c.nlines, stats=True)   # geometry and tables cached
        t2 = time.perf_counter()
        t_cold += t1 - t0
        t_warm += t2 - t1
        rc_total += st["ray_channels"]
        plain.append(f)
        m.free()
    # batched: all jobs resident, one geometry + walk + reduction per memory wave, graph replay
    models = [ctx.load_arrays(synth.model_arrays(c), cam) for c, cam in zip(cfgs, cams)]
    b = rl.Batch(ctx)
    for c, m in zip(cfgs, models):
        b.add(m, c.ilinestart, c.nlines)
    t0 = time.perf_counter()
    tune = b.autotune(sample_stride=tune_stride)
    t_setup = time.perf_counter() - t0
    b.run()                                                  # graph capture + first replay
    times, walls = [], []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        out, st = b.run(stats=True)
        walls.append(time.perf_counter() - t0)
        times.append(st["total_ms"] * 1e-3)
    rel = 0.0
    for got, ref in zip(out, plain):
        for k in range(ref.shape[0]):
            sel = ref[k] > 1e-3 * ref[k].max()
            if sel.any():
                rel = max(rel, float(np.max(np.abs(got[k][sel] - ref[k][sel]) / np.abs(ref[k][sel]))))
    t_b = statistics.median(times)
    res = {"workload": f"{n_models} uneven disks (nr 64-512, ntheta 32-256, 1-50 lines, 32-256 channels, "
                       f"incl 5-85 deg, {cfgs[0].nphi} azimuths)",
           "spectra": nspec, "ray_channels": rc_total,
           "plain": {"s_cold": t_cold, "s_warm": t_warm, "spectra_per_s_warm": nspec / t_warm,
                     "spectra_per_s_cold": nspec / t_cold, "ray_channels_per_s_warm": rc_total / t_warm},
           "batched": {"s": t_b, "wall_s": statistics.median(walls), "spectra_per_s": nspec / t_b,
                       "ray_channels_per_s": rc_total / t_b, "tiles": tune, "tune_s": t_setup,
                       "waves": b.waves(), "graph": True},
           "speedup_vs_plain_warm": t_warm / t_b, "speedup_vs_plain_cold": t_cold / t_b,
           "max_rel_diff_batched_vs_plain": rel}
    b.close()
    for m in models:
        m.free()
    return res


def adjoint_case(ctx, name="adjoint_disk", reps=3, **over):
    """Forward and forward+adjoint of the differentiable raytrace (per-cell ln T, ln X,
    width) on one model, FP32; timed with the library's CUDA events."""
    import numpy as np
    import torch
    import radlite_gb300 as rl
    from radlite_gb300 import synth
    cfg = synth.config_by_name(name, **over)
    m = ctx.load_arrays(synth.lte_arrays(cfg), camera(cfg, cfg.incl_deg))
    lnT, lnX, b = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in synth.cell_params(cfg))
    d = rl.Diff(m, cfg.ilinestart, cfg.nlines, precision=0)
    target = d.forward(lnT + 0.05, lnX, b)
    fw, bw = [], []
    for _ in range(reps + 1):
        flux, st = d.forward(lnT, lnX, b, stats=True)
        gflux = 2.0 * (flux - target) / target.abs().max() ** 2
        _, sb = d.backward(gflux, stats=True)
        fw.append(st["total_ms"])
        bw.append(sb["total_ms"])
    res = {"workload": f"{name}: {cfg.nr}x{cfg.nt} disk, {cfg.nlines} lines x {d.nfr} channels, {d.nrays} rays, "
                       "gradients w.r.t. per-cell ln T, ln X, width",
           "forward_ms": statistics.median(fw[1:]), "adjoint_ms": statistics.median(bw[1:]),
           "spectra": cfg.nlines}
    # the reverse sweep over stored intensities (checkpoint interval 1), whose forward is the
    # plain walk (the gradient sweep's forward also keeps each channel's optical depth)
    d.set_checkpoint(1)
    fp = []
    for _ in range(2):
        flux, sf = d.forward(lnT, lnX, b, stats=True)
        fp.append(sf["total_ms"])
    gflux = 2.0 * (flux - target) / target.abs().max() ** 2
    rv = []
    for _ in range(2):
        _, sb = d.backward(gflux, stats=True)
        rv.append(sb["total_ms"])
    d.set_checkpoint(0)
    res["forward_plain_walk_ms"] = min(fp)
    res["reverse_sweep_ms"] = min(rv)
    res["adjoint_over_forward"] = res["adjoint_ms"] / res["forward_ms"]
    res["forward_adjoint_over_plain_forward"] = (res["forward_ms"] + res["adjoint_ms"]) / res["forward_plain_walk_ms"]
    res["forward_adjoint_spectra_per_s"] = cfg.nlines / ((res["forward_ms"] + res["adjoint_ms"]) * 1e-3)
    # the same gradient by central differences: two forwards per cell parameter
    npar = 3 * int(lnT.numel())
    res["parameters"] = npar
    res["speedup_vs_central_differences"] = ((2 * npar + 1) * res["forward_ms"]
                                             / (res["forward_ms"] + res["adjoint_ms"]))
    d.close()
    m.free()
    return res


def fit_case(ctx, n_models=64, steps=5, plain_models=8, nphi=32, dbdr=2, history=False, analyse=False):
    """The batched forward+adjoint fitting step on n uneven models (radlite_gb300.fit)
    against plain per-model forward + central finite differences in the four parameters,
    timed on `plain_models` of the same models."""
    from radlite_gb300 import fit
    cfgs = fit.fit_configs(n_models, nphi=nphi, dbdr=dbdr)
    res = fit.run_fit(ctx, cfgs, steps=steps, history=history, analyse=analyse)
    plain = fit.plain_fd_step_seconds(ctx, cfgs[:plain_models])
    per_spec = plain["seconds"] / plain["spectra"]
    out = {"workload": f"{n_models} uneven disks (nr 100-400, ntheta 50-200), 20 lines x 200 channels, "
                       f"{cfgs[0].nphi} azimuths, {dbdr} rings per grid radius, 4 parameters each",
           "batched_forward_adjoint": res,
           "plain_forward_fd": {"models_timed": plain_models, "seconds_per_gradient_spectrum": per_spec,
                                "spectra_per_s": 1.0 / per_spec}}
    out["speedup_vs_plain_fd"] = res["forward_adjoint_spectra_per_s"] * per_spec
    # four parameters: central differences cost 9 forwards per gradient, the batched
    # forward + adjoint this many forwards' time
    out["forward_equivalents_per_gradient"] = ((res["forward_ms_per_step"] + res["adjoint_ms_per_step"])
                                               / res["forward_ms_per_step"])
    return out


def recovery_case(ctx, n_models=8, steps=200, nphi=8, dbdr=1):
    """Parameter recovery of the fitting loop: `steps` Adam steps on n uneven disks of the
    fitting workload (smaller images, so that 200 steps stay within a minute or two), the
    error of each parameter every 10 steps, and the Gauss-Newton eigen-analysis at the end
    point (which parameter combinations the spectra constrain)."""
    from radlite_gb300 import fit
    cfgs = fit.fit_configs(n_models, nphi=nphi, dbdr=dbdr)
    res = fit.run_fit(ctx, cfgs, steps=steps, history=True, analyse=True)
    res["workload"] = (f"{n_models} uneven disks (nr 100-400, ntheta 50-200), 20 lines x 200 channels, {nphi} "
                       f"azimuths, {dbdr} ring per grid radius, 4 parameters each, {steps} Adam steps (lr 0.02)")
    return res


def profile_case(args):
    """One pass of a named workload (geometry, walk, reduction), for profiler captures.
    "posvel_disk": the 200x100 disk's 128x128-pixel position-velocity cube of 2 lines;
    "genspec_band": gen_spec of 500 lines x 201 channels; "adjoint_grad": forward and
    backward of the differentiable 200x100 disk, both adjoint modes."""
    import numpy as np
    import radlite_gb300 as rl
    from radlite_gb300 import synth
    if args.workload == "genspec_band":
        rng = np.random.default_rng(5)
        vel = np.linspace(-20.0, 20.0, 201)
        lines = [{"vel": vel, "flux": (1 + 0.001 * vel) * rng.uniform(1e-20, 2e-20)
                  + rng.uniform(0, 4e-20) * np.exp(-(vel / rng.uniform(2, 6)) ** 2),
                  "freq": 2.99792458e10 * rng.uniform(2000.0, 2050.0), "maxnumpoints": 201} for _ in range(500)]
        ctx = rl.Context(0)
        o = ctx.gen_spec(lines, 3.0, 1.0, 140.0, stats=True)
        print(json.dumps({"workload": args.workload, "fine_points": o["stats"]["nrays"],
                          "device_ms": o["stats"]["walk_ms"]}), flush=True)
        ctx.close()
        return 0
    if args.workload == "posvel_disk":
        cfg = synth.config_by_name("adjoint_disk")
        arr = synth.model_arrays(cfg)
        ctx = rl.Context(0)
        m = ctx.load_arrays(arr, camera(cfg, cfg.incl_deg))
        size = 2.0 * float(arr["r"][-1])
        m.set_posvel(128, 128, size, size, addstar=1)
        _, _, st = m.posvel(cfg.ilinestart, 2, stats=True)
        print(json.dumps({"workload": args.workload, "steps": st["steps"], "walk_ms": st["walk_ms"],
                          "geometry_ms": st["geometry_ms"], "nrays": st["nrays"], "ray_channels": st["ray_channels"]}),
              flush=True)
        m.free()
        ctx.close()
        return 0
    if args.workload == "adjoint_grad":
        # one differentiable forward and one backward of the 200x100 disk per adjoint mode:
        # the gradient sweep (checkpoint interval 0), then the reverse sweep (interval 1)
        import torch
        cfg = synth.config_by_name("adjoint_disk", **({"nphi": args.nphi} if args.nphi else {}))
        ctx = rl.Context(0)
        m = ctx.load_arrays(synth.lte_arrays(cfg), camera(cfg, cfg.incl_deg))
        lnT, lnX, b = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in synth.cell_params(cfg))
        d = rl.Diff(m, cfg.ilinestart, cfg.nlines, precision=0)
        target = d.forward(lnT + 0.05, lnX, b)
        flux, fst = d.forward(lnT, lnX, b, stats=True)
        gflux = 2.0 * (flux - target) / target.abs().max() ** 2
        out = {"workload": args.workload, "nrays": d.nrays, "forward_ms": fst["total_ms"]}
        for every in (0, 1):
            d.set_checkpoint(every)
            d.forward(lnT, lnX, b)      # each adjoint mode differentiates a forward of its own
            _, st = d.backward(gflux, stats=True)
            out[f"interval_{every}"] = {k: st[k] for k in ("total_ms", "steps", "refined_passes", "refined_channels")}
        print(json.dumps(out), flush=True)
        d.close()
        m.free()
        ctx.close()
        return 0
    cfg = synth.config_by_name(args.workload, **({"nphi": args.nphi} if args.nphi else {}))
    arr = synth.model_arrays(cfg)
    ctx = rl.Context(0)
    m = ctx.load_arrays(arr, camera(cfg, cfg.incl_deg))
    f, st = m.spectra(cfg.ilinestart, cfg.nlines, stats=True)
    print(json.dumps({"workload": args.workload, "steps": st["steps"], "walk_ms": st["walk_ms"],
                      "geometry_ms": st["geometry_ms"], "nrays": st["nrays"], "nlines": st["nlines"],
                      "node_passes": st["node_passes"], "packed_passes": st["packed_passes"],
                      "empty_steps": st["empty_steps"], "refined_passes": st["refined_passes"],
                      "sub_steps": st["sub_steps"]}), flush=True)
    m.free()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--profile", action="store_true", help="one pass of --workload (profiler captures)")
    ap.add_argument("--workload", default="adjoint_disk")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-stride", type=int, default=32,
                    help="ray stride of the oracle sample (CPU baseline and parity): all lines, both inclinations")
    ap.add_argument("--ref-stride", type=int, default=509,
                    help="ray stride of each step of --impl reference (all lines, both inclinations)")
    ap.add_argument("--fit-steps", type=int, default=3, help="Adam steps of the fitting measurement")
    ap.add_argument("--recovery-steps", type=int, default=200,
                    help="Adam steps of the parameter-recovery study (0 skips it)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-verify", action="store_true")
    ap.add_argument("--batch-models", type=int, default=256,
                    help="models of the uneven batched comparison (0 skips it)")
    ap.add_argument("--only-batch", action="store_true", help="run only the batched comparison")
    ap.add_argument("--only-adjoint", action="store_true", help="run only the forward+adjoint timing")
    ap.add_argument("--nphi", type=int, default=0,
                    help="azimuths of the adjoint timing and of --profile (0: the workload's)")
    ap.add_argument("--only-fit", action="store_true", help="run only the batched fitting-step comparison")
    ap.add_argument("--only-recovery", action="store_true", help="run only the parameter-recovery study")
    ap.add_argument("--fit-models", type=int, default=16)
    ap.add_argument("--fit-nphi", type=int, default=32, help="azimuths of the fitting images")
    ap.add_argument("--fit-dbdr", type=int, default=2, help="rings per grid radius of the fitting images")
    ap.add_argument("--no-diff", action="store_true", help="skip the adjoint and fitting measurements")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the position-velocity, gen_spec and input-parsing measurements")
    args = ap.parse_args()
    if args.only_recovery:
        import radlite_gb300 as rl
        ctx = rl.Context(0)
        print(json.dumps(recovery_case(ctx, steps=args.recovery_steps)), flush=True)
        ctx.close()
        return 0
    if args.only_fit:
        import radlite_gb300 as rl
        ctx = rl.Context(0)
        print(json.dumps(fit_case(ctx, args.fit_models, args.fit_steps, nphi=args.fit_nphi, dbdr=args.fit_dbdr,
                                  history=True, analyse=True, plain_models=min(8, args.fit_models))), flush=True)
        ctx.close()
        return 0
    if args.only_adjoint:
        import radlite_gb300 as rl
        ctx = rl.Context(0)
        over = {"nphi": args.nphi} if args.nphi else {}
        print(json.dumps(adjoint_case(ctx, **over)), flush=True)
        ctx.close()
        return 0
    if args.only_batch:
        import radlite_gb300 as rl
        ctx = rl.Context(0)
        print(json.dumps(batched_case(ctx, args.batch_models, args.steps)), flush=True)
        ctx.close()
        return 0
    if args.warmup < 3:
        args.warmup = 3
    if args.profile:
        return profile_case(args)
    return reference_arm(args) if args.impl == "reference" else ours(args)


if __name__ == "__main__":
    sys.exit(main())
