"""Batched forward+adjoint fitting of parametric disk models to line spectra.

Each model has four free parameters of the synthetic disk laws (radlite_gb300.synth):
ln T0 and the index q of the temperature law T = T0 (r / 0.1 AU)^q, the molecular
abundance ln X0, and ln f of the turbulent width b = sqrt((f c_s)^2 + 2kT/m). Every step
renders all models' spectra with one forward and one adjoint launch sequence (DiffBatch,
replayed from CUDA graphs), maps the per-cell gradients to the four parameters with torch
autograd, and takes an Adam step. The targets are the spectra of seeded "true"
parameters; the fit starts from a seeded offset.

The reference has no fitting path (pyradlite runs the Fortran once per model and
post-processes, radlite.py:592-595); the forward it differentiates is the line raytrace of
calc_line_spectrum (main.F:1043-1049).
"""
from __future__ import annotations

import math
import time
from dataclasses import replace

import numpy as np

from . import synth

PARAMS = ("lnT0", "q", "lnX0", "lnf")


def fit_configs(n: int = 64, seed: int = 4, nphi: int = 4, nlines: int = 20, nch: int = 200, dbdr: int = 1) -> list:
    """n uneven disks: nr ~ U[100,400], ntheta ~ U[50,200], 20 ro-vibrational lines x 200
    channels, inclination ~ U[5,85] deg, stellar mass ~ U[0.3,2.5] Msun; nphi azimuths and
    dbdr rings per grid radius."""
    rng = np.random.default_rng(seed)
    out = []
    dv = 0.25
    for i in range(n):
        nr = int(rng.integers(100, 401))
        nt = int(rng.integers(50, 201))
        out.append(synth.DiskConfig(
            name=f"fit{i:02d}", nr=nr, nt=nt, mstar=float(rng.uniform(0.3, 2.5)),
            incl_deg=float(rng.uniform(5.0, 85.0)), molecule="band", band_nj=nlines // 2, ilinestart=1,
            nlines=nlines, dv=dv, vmax=((nch - 1) + 0.05) * dv / 2.0, nphi=nphi, dbdr=dbdr,
            nrrextra=-max(8, nr // 8), seed=seed * 1000 + i))
    return out


def true_params(cfg) -> np.ndarray:
    return np.array([math.log(cfg.t0), cfg.t_pow, math.log(cfg.abund), math.log(cfg.turb_frac)])


def with_params(cfg, p):
    return replace(cfg, t0=float(math.exp(p[0])), t_pow=float(p[1]), abund=float(math.exp(p[2])),
                   turb_frac=float(math.exp(p[3])))


class DiskFit:
    """The fitting problem: models loaded at the starting parameters, targets rendered at
    the true ones."""

    def __init__(self, ctx, cfgs, offset=(0.15, 0.08, -0.4, 0.4), precision: int = 0, seed: int = 5):
        import torch
        import radlite_gb300 as rl
        self.ctx, self.cfgs = ctx, cfgs
        rng = np.random.default_rng(seed)
        self.p_true = torch.tensor(np.stack([true_params(c) for c in cfgs]), dtype=torch.float64, device="cuda")
        off = np.asarray(offset) * rng.uniform(0.5, 1.0, size=(len(cfgs), 4))
        self.p0 = self.p_true + torch.tensor(off, dtype=torch.float64, device="cuda")
        self.models, self.diffs, self.geo = [], [], []
        self.batch = rl.DiffBatch(ctx)
        for c, p in zip(cfgs, self.p0.cpu().numpy()):
            c0 = with_params(c, p)          # the loaded model knows only the starting guess
            cam = dict(incl_deg=c.incl_deg, nphi=c.nphi, dbdr=c.dbdr, nrrayextra=c.nrrextra, vmax=c.vmax, dv=c.dv,
                       ilinestart=c.ilinestart, nlines=c.nlines)
            m = ctx.load_arrays(synth.lte_arrays(c0), cam)
            d = rl.Diff(m, c.ilinestart, c.nlines, precision=precision)
            self.models.append(m)
            self.diffs.append(d)
            self.batch.add(d)
            r, _ = synth.make_grid(c)
            lnr = np.repeat(np.log(r / (c.t_r0_au * synth.AU)), c.nt)         # cell order (ir-1)*nth + (it-1)
            self.geo.append(torch.tensor(lnr, dtype=torch.float64, device="cuda"))
        kb = synth.KB
        self.alpha = 1.4 * kb / (2.3 * synth.MP)
        self.beta = [2.0 * kb / (c.mol_mass_amu * synth.AMU) for c in cfgs]
        self.views = self.batch.tensors()
        self.target = None

    def cell_fields(self, p):
        """Per-model (ln T, ln X, width) cell arrays as torch functions of p [n, 4]."""
        out = []
        for j, lnr in enumerate(self.geo):
            lnT = p[j, 0] + p[j, 1] * lnr
            lnX = p[j, 2] + 0.0 * lnr
            T = lnT.exp()
            f2 = (2.0 * p[j, 3]).exp()
            b = (T * (self.alpha * f2 + self.beta[j])).sqrt() / 1.0e5
            out.append((lnT, lnX, b))
        return out

    def _load(self, fields):
        for v, (lnT, lnX, b) in zip(self.views["models"], fields):
            v["lnT"].copy_(lnT.detach())
            v["lnX"].copy_(lnX.detach())
            v["width"].copy_(b.detach())

    def render(self, p):
        import torch
        with torch.no_grad():
            self._load(self.cell_fields(p))
        self.batch.forward()
        return [v["flux"].clone() for v in self.views["models"]]

    def set_target(self):
        self.target = self.render(self.p_true)
        self.tnorm = [float((t * t).sum()) for t in self.target]

    def loss_and_grad(self, p):
        """Sum over models of |F - F_target|^2 / |F_target|^2 and its gradient in p."""
        import torch
        fields = self.cell_fields(p)
        with torch.no_grad():
            self._load(fields)
        fst = self.batch.forward(stats=True)
        loss = 0.0
        with torch.no_grad():
            for v, t, tn in zip(self.views["models"], self.target, self.tnorm):
                r = v["flux"] - t
                loss += float((r * r).sum()) / tn
                v["gflux"].copy_(2.0 * r / tn)
        bst = self.batch.backward(stats=True)
        tens, grads = [], []
        for (lnT, lnX, b), v in zip(fields, self.views["models"]):
            tens += [lnT, lnX, b]
            grads += [v["g_lnT"].clone(), v["g_lnX"].clone(), v["g_width"].clone()]
        g, = torch.autograd.grad(tens, [p], grads)
        return loss, g, fst, bst

    def close(self):
        self.batch.close()
        for d in self.diffs:
            d.close()
        for m in self.models:
            m.free()


def gauss_newton(fit, p, rel: float = 1e-3) -> dict:
    """Which parameter combinations the spectra constrain at p: per model the Jacobian J of
    its normalised spectra (F / |F_target|) in the four parameters, by central differences
    of the batched forward (each parameter moved in every model at once: a model's spectra
    depend on its own parameters only), and the eigenvalues of J^T J, the Gauss-Newton
    Hessian of the loss. A small eigenvalue marks a combination the spectra hardly change
    with (a degeneracy); its eigenvector names the combination. "vectors" holds each model's
    eigenvectors as columns, weakest first."""
    import torch
    cols = []
    for k in range(4):
        q = p.detach().clone()
        q[:, k] += rel
        fp = fit.render(q)
        q[:, k] -= 2 * rel
        fm = fit.render(q)
        cols.append([((a - b) / (2 * rel)).flatten() / math.sqrt(tn) for a, b, tn in zip(fp, fm, fit.tnorm)])
    out = {"eigenvalues": [], "weakest_direction": [], "condition": [], "vectors": []}
    for j in range(len(fit.cfgs)):
        J = torch.stack([cols[k][j] for k in range(4)], dim=1)
        ev, vec = torch.linalg.eigh(J.T @ J)
        ev = ev.cpu().numpy()
        out["eigenvalues"].append([float(x) for x in ev])
        out["weakest_direction"].append([float(x) for x in vec[:, 0].cpu().numpy()])
        out["vectors"].append(vec.cpu().numpy().tolist())
        out["condition"].append(float(ev[-1] / max(ev[0], 1e-300)))
    return out


def error_in_eigenbasis(gn: dict, e_start, e_end) -> dict:
    """The parameter error of each model at the start and the end of a fit, split over the
    eigenvectors of its end-point Gauss-Newton Hessian H = J^T J: the component along the
    weakest eigenvector (the combination the spectra hardly constrain) and the error the
    spectra do see, sqrt(e^T H e) (the first-order change of the normalised spectra, in
    units of the loss's norm). A fit that reduces the second while the first stays put or
    grows has recovered everything the spectra determine."""
    out = {"weak_component_start": [], "weak_component_end": [], "seen_error_start": [], "seen_error_end": []}
    for j, (ev, vec) in enumerate(zip(gn["eigenvalues"], gn["vectors"])):
        v = np.asarray(vec)
        lam = np.asarray(ev)
        for tag, e in (("start", e_start[j]), ("end", e_end[j])):
            c = v.T @ e
            out[f"weak_component_{tag}"].append(float(c[0]))
            out[f"seen_error_{tag}"].append(float(math.sqrt(max(float(np.sum(lam * c * c)), 0.0))))
    out["median_seen_error_ratio_end_over_start"] = float(np.median(
        np.asarray(out["seen_error_end"]) / np.maximum(np.asarray(out["seen_error_start"]), 1e-300)))
    return out


def run_fit(ctx, cfgs, steps: int = 200, lr: float = 0.02, precision: int = 0, log=None, history: bool = False,
            analyse: bool = False) -> dict:
    """Adam on all models at once; returns throughput and parameter recovery (with
    history=True the largest error of each parameter every 10 steps; with analyse=True the
    Gauss-Newton eigen-analysis at the end point)."""
    import torch
    fit = DiskFit(ctx, cfgs, precision=precision)
    fit.set_target()
    p = fit.p0.clone().requires_grad_(True)
    opt = torch.optim.Adam([p], lr=lr)
    err0 = (fit.p0 - fit.p_true).abs().max(dim=0).values.cpu().numpy()
    fw_ms = bw_ms = 0.0
    t0 = time.perf_counter()
    losses, hist = [], []
    for it in range(steps):
        loss, g, fst, bst = fit.loss_and_grad(p)
        fw_ms += fst["total_ms"]
        bw_ms += bst["total_ms"]
        opt.zero_grad()
        p.grad = g
        opt.step()
        losses.append(loss)
        if history and (it % 10 == 0 or it == steps - 1):
            e = (p.detach() - fit.p_true).abs()
            hist.append({"step": it + 1, "loss": loss, "max_abs_error": dict(zip(PARAMS, map(float, e.max(dim=0).values))),
                         "median_abs_error": dict(zip(PARAMS, map(float, e.median(dim=0).values)))})
        if log and (it % 20 == 0 or it == steps - 1):
            log(f"step {it} loss {loss:.4e}")
    wall = time.perf_counter() - t0
    err = (p.detach() - fit.p_true).abs().max(dim=0).values.cpu().numpy()
    errm = (p.detach() - fit.p_true).abs().median(dim=0).values.cpu().numpy()
    nspec = sum(c.nlines for c in cfgs)
    res = {"models": len(cfgs), "steps": steps, "spectra_per_step": nspec,
           "loss_first": losses[0], "loss_last": losses[-1],
           "forward_ms_per_step": fw_ms / steps, "adjoint_ms_per_step": bw_ms / steps,
           "wall_s": wall, "forward_adjoint_spectra_per_s": nspec * steps / ((fw_ms + bw_ms) * 1e-3),
           "wall_spectra_per_s": nspec * steps / wall,
           "max_abs_param_error_start": dict(zip(PARAMS, map(float, err0))),
           "max_abs_param_error_end": dict(zip(PARAMS, map(float, err))),
           "median_abs_param_error_end": dict(zip(PARAMS, map(float, errm)))}
    if history:
        res["history"] = hist
    if analyse:
        gn = gauss_newton(fit, p)
        res["gauss_newton"] = gn
        res["error_in_eigenbasis"] = error_in_eigenbasis(gn, (fit.p0 - fit.p_true).cpu().numpy(),
                                                         (p.detach() - fit.p_true).cpu().numpy())
    fit.close()
    return res


def plain_fd_step_seconds(ctx, cfgs, precision: int = 0) -> dict:
    """One gradient step the plain way for each model: a per-model forward launch plus
    central finite differences in the four parameters (9 forwards per model), with the
    model's tables rebuilt on the host from the loaded populations each time."""
    import radlite_gb300 as rl
    t = 0.0
    nspec = 0
    for c in cfgs:
        p = true_params(c)
        for k in range(9):
            q = p.copy()
            if k > 0:
                q[(k - 1) // 2] += 1e-4 * (1 if k % 2 else -1)
            cq = with_params(c, q)
            cam = dict(incl_deg=c.incl_deg, nphi=c.nphi, dbdr=c.dbdr, nrrayextra=c.nrrextra, vmax=c.vmax, dv=c.dv,
                       ilinestart=c.ilinestart, nlines=c.nlines)
            arr = synth.lte_arrays(cq)
            m = ctx.load_arrays(arr, cam)
            m.set_precision(precision)
            t0 = time.perf_counter()
            m.spectra(c.ilinestart, c.nlines)
            t += time.perf_counter() - t0
            m.free()
        nspec += c.nlines
    return {"seconds": t, "spectra": nspec, "spectra_per_s": nspec / t}
