"""The adjoint at the adjoint workload's grid and against the oracle's finite differences.

* adjoint_disk: the 200x100 disk with 10 lines x 128 channels (600 rings; 8 azimuths instead
  of 128, so that a few hundred FP64 forwards stay within seconds). FP64 adjoint against
  FP64 central differences of the same forward, relative step 1e-4 (1e-6 where a kink of
  the piecewise forward lies within the step), on at least 32 random cells per parameter
  among those whose gradient exceeds 1e-4 of the largest: <= 1e-3 relative.
* tiny_band against the oracle: the reference formats written with the cell's parameter
  moved by +-h (LTE level populations and dust temperature for ln T, abundance.inp for
  ln X, turbulence.inp for the width), rendered by the FP64 oracle in host processes; its
  central difference of the linear loss sum(gflux * F) against the GPU's FP64 adjoint at
  the same gflux: <= 1e-3 relative on at least 32 cells per parameter whose +-h renders
  keep the base render's discrete decisions (step and integrated-channel counts); relative
  step 1e-4, then 1e-5 and 1e-6 where a kink of the piecewise forward lies within the
  larger step.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FD_TOL = 1e-3


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _model(gpu_lib, ctx, cfg):
    import torch
    from radlite_gb300 import synth
    cam = dict(incl_deg=cfg.incl_deg, nphi=cfg.nphi, dbdr=cfg.dbdr, nrrayextra=cfg.nrrextra, vmax=cfg.vmax,
               dv=cfg.dv, ilinestart=cfg.ilinestart, nlines=cfg.nlines)
    m = ctx.load_arrays(synth.lte_arrays(cfg), cam)
    lnT, lnX, b = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in synth.cell_params(cfg))
    return m, lnT, lnX, b


def test_adjoint_fd_adjoint_disk(gpu_lib, ctx):
    from radlite_gb300 import synth
    cfg = synth.config_by_name("adjoint_disk", nphi=8)
    m, lnT, lnX, b = _model(gpu_lib, ctx, cfg)
    d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
    assert d.nfr == 128
    target = d.forward(lnT + 0.05, lnX, b * 1.05)
    flux, st0 = d.forward(lnT, lnX, b, stats=True)
    base = (st0["steps"], st0["integrated"])
    scale = target.abs().max()
    gflux = 2.0 * (flux - target) / scale ** 2
    grads = [g.cpu().numpy() for g in d.backward(gflux)]
    params = {"lnT": lnT, "lnX": lnX, "width": b}

    def loss(f):
        return float((((f - target) / scale) ** 2).sum())

    def central(name, c, rel):
        h = rel if name != "width" else rel * float(b[c])
        vals, same = [], True
        for sgn in (1.0, -1.0):
            q = {k: v.clone() for k, v in params.items()}
            q[name][c] += sgn * h
            f, st = d.forward(q["lnT"], q["lnX"], q["width"], stats=True)
            same = same and (st["steps"], st["integrated"]) == base
            vals.append(loss(f))
        return (vals[0] - vals[1]) / (2 * h), same

    rng = np.random.default_rng(5)
    report = {}
    for name, g in zip(("lnT", "lnX", "width"), grads):
        cand = rng.permutation(np.flatnonzero(np.abs(g) > 1e-4 * np.abs(g).max()))
        errs = []
        for c in cand[:120]:
            if len(errs) == 40:
                break
            fd, same = central(name, c, 1e-4)
            if not same:
                continue
            err = abs(fd - g[c]) / max(abs(fd), 1e-300)
            if err > FD_TOL:
                fd, same = central(name, c, 1e-6)
                if not same:
                    continue
                err = abs(fd - g[c]) / max(abs(fd), 1e-300)
            errs.append(err)
        report[name] = (len(errs), float(np.max(errs)) if errs else None, float(np.median(errs)) if errs else None)
    for name, (n, mx, _) in report.items():
        assert n >= 32, report
        assert mx <= FD_TOL, report
    d.close()
    m.free()


def test_adjoint_vs_oracle_finite_differences(gpu_lib, ctx, oracle_lib):
    import multiprocessing as mp
    from radlite_gb300 import synth
    cfg = synth.config_by_name("tiny_band")
    m, lnT, lnX, b = _model(gpu_lib, ctx, cfg)
    p0 = [t.cpu().numpy() for t in (lnT, lnX, b)]
    from oracle import sample
    f0, steps0, integ0 = sample.render_params(("tiny_band", *p0))
    d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
    fg = d.forward(lnT, lnX, b).cpu().numpy()
    sel = f0 > 1e-3 * f0.max(axis=1, keepdims=True)
    assert np.max(np.abs(fg[sel] - f0[sel]) / f0[sel]) <= 1e-5   # the same model on both sides
    rng = np.random.default_rng(9)
    wts = rng.uniform(0.5, 1.5, f0.shape) / np.abs(f0).max()
    import torch
    grads = [g.cpu().numpy() for g in d.backward(torch.tensor(wts, dtype=torch.float64, device="cuda"))]
    names = ("lnT", "lnX", "width")
    cells = [rng.permutation(np.flatnonzero(np.abs(g) > 1e-3 * np.abs(g).max()))[:56] for g in grads]

    def fd_round(picks, h, pool):
        jobs, keys = [], []
        for pi, c in picks:
            step = h if names[pi] != "width" else h * p0[2][c]
            for sgn in (1.0, -1.0):
                q = [a.copy() for a in p0]
                q[pi][c] += sgn * step
                jobs.append(("tiny_band", *q))
            keys.append((pi, c, step))
        res = pool.map(sample.render_params, jobs)
        out = {}
        for i, (pi, c, step) in enumerate(keys):
            (fp, sp, ip), (fm, sm, im) = res[2 * i], res[2 * i + 1]
            if (sp, ip) != (steps0, integ0) or (sm, im) != (steps0, integ0):
                continue                  # a discrete decision moved within +-h
            fd = float(np.sum(wts * (fp - fm))) / (2 * step)
            out[(pi, c)] = abs(fd - grads[pi][c]) / max(abs(fd), 1e-300)
        return out

    # relative step 1e-4; where that difference disagrees (a kink of the piecewise forward,
    # e.g. the source bracket switching or a sub-step moving, within +-h) again at 1e-5 and
    # 1e-6, which the text formats still resolve for the temperature and the width (not for
    # the abundance's 9 digits, whose differences agree at 1e-4)
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        first = fd_round([(pi, c) for pi in range(3) for c in cells[pi]], 1e-4, pool)
        again = dict(first)
        for h in (1e-5, 1e-6):
            redo = [k for k, e in again.items() if e > FD_TOL and names[k[0]] != "lnX"]
            if not redo:
                break
            finer = fd_round(redo, h, pool)
            for k in redo:
                if k in finer:
                    again[k] = finer[k]
                else:
                    again.pop(k)          # the finer step met a decision change
    report = {n: [] for n in names}
    worst = []
    for (pi, c), e in again.items():
        report[names[pi]].append(e)
        worst.append((e, pi, int(c)))
    summary = {n: (len(e), max(e) if e else None) for n, e in report.items()}
    bad = [w for w in sorted(worst)[-4:] if w[0] > FD_TOL]
    if bad:
        # the same central difference of the GPU's own FP64 forward, for the message
        params = [lnT, lnX, b]
        for e, pi, c in bad:
            step = 1e-6 if names[pi] != "width" else 1e-6 * p0[2][c]
            vals = []
            for sgn in (1.0, -1.0):
                q = [t.clone() for t in params]
                q[pi][c] += sgn * step
                vals.append(float((torch.tensor(wts, device="cuda") * d.forward(*q)).sum()))
            summary[f"{names[pi]} cell {c}"] = {"rel_err": e, "adjoint": float(grads[pi][c]),
                                                 "gpu_fd": (vals[0] - vals[1]) / (2 * step)}
    for n in names:
        cnt, mx = summary[n]
        assert cnt >= 32, summary
        assert mx <= FD_TOL, summary
    d.close()
    m.free()
