"""The differentiable raytrace (rl_diff_*): LTE tables on the device, the adjoint walk,
and the torch.autograd binding.

* forward: with LTE populations on both sides, the differentiable forward equals the
  plain path's spectra (FP64 <= 1e-10, FP32 <= 1e-5 relative in channels above 1e-3 of
  the peak);
* gradient: the FP64 adjoint against FP64 central finite differences of the same forward
  (relative step 1e-4) on 64 random cells per parameter, <= 1e-3 relative;
* FP32 adjoint against the FP64 adjoint: relative L2 difference <= 1e-2, <= 5e-2 on any
  cell above 1e-2 of the largest gradient."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FD_TOL = 1e-3


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _setup(gpu_lib, ctx, name="tiny_band", **over):
    import torch
    from radlite_gb300 import synth
    cfg = synth.config_by_name(name, **over)
    arr = synth.lte_arrays(cfg)
    cam = dict(incl_deg=cfg.incl_deg, nphi=cfg.nphi, dbdr=cfg.dbdr, nrrayextra=cfg.nrrextra, vmax=cfg.vmax,
               dv=cfg.dv, ilinestart=cfg.ilinestart, nlines=cfg.nlines)
    m = ctx.load_arrays(arr, cam)
    lnT, lnX, b = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in synth.cell_params(cfg))
    return cfg, m, lnT, lnX, b


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


@pytest.mark.parametrize("prec,tol", [(1, 1e-10), (0, 1e-5)])
def test_diff_forward_matches_plain_path(gpu_lib, ctx, prec, tol):
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx)
    m.set_precision(prec)
    ref = m.spectra(cfg.ilinestart, cfg.nlines)
    d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=prec)
    got = d.forward(lnT, lnX, b).cpu().numpy()
    for k in range(cfg.nlines):
        assert relerr(got[k], ref[k]) <= tol, (k, relerr(got[k], ref[k]))
    d.close()
    m.free()


def _loss(flux, target):
    return float((((flux - target) / target.abs().max()) ** 2).sum())


def test_adjoint_matches_central_differences(gpu_lib, ctx):
    """Cells are drawn at random among those with a gradient above 1e-4 of the largest.
    The forward is piecewise smooth: the SUBGRID sub-step grid moves with the line width,
    and the source-term bracket switches. A cell counts when its +-h forwards keep the base
    forward's discrete decisions (formal-solution step count, integrated channels). The
    central difference uses relative step 1e-4; where a kink lies within +-h (the 1e-4
    difference disagrees), the step is cut to 1e-6 so that it stays on the smooth piece,
    and the adjoint must agree with that."""
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx)
    d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
    # target: the same disk 5% warmer, 20% more abundant, 10% broader lines
    target = d.forward(lnT + 0.05, lnX + np.log(1.2), b * 1.1)
    flux, st0 = d.forward(lnT, lnX, b, stats=True)
    base = (st0["steps"], st0["integrated"])
    scale = target.abs().max()
    gflux = 2.0 * (flux - target) / scale ** 2
    gT, gX, gb = d.backward(gflux)
    rng = np.random.default_rng(11)
    params = {"lnT": lnT, "lnX": lnX, "width": b}

    def central(name, c, rel):
        h = rel if name != "width" else rel * float(b[c])
        vals, same = [], True
        for sgn in (1.0, -1.0):
            q = {k: v.clone() for k, v in params.items()}
            q[name][c] += sgn * h
            f, st = d.forward(q["lnT"], q["lnX"], q["width"], stats=True)
            same = same and (st["steps"], st["integrated"]) == base
            vals.append(_loss(f, target))
        return (vals[0] - vals[1]) / (2 * h), same

    report = {}
    for name, g in (("lnT", gT), ("lnX", gX), ("width", gb)):
        g = g.cpu().numpy()
        big = rng.permutation(np.flatnonzero(np.abs(g) > 1e-4 * np.abs(g).max()))
        errs, tried, refined = [], 0, 0
        for c in big:
            if len(errs) == 64 or tried == 160:
                break
            tried += 1
            fd, same = central(name, c, 1e-4)
            if not same:
                continue
            err = abs(fd - g[c]) / max(abs(fd), 1e-30)
            if err > FD_TOL:
                fd, same = central(name, c, 1e-6)
                if not same:
                    continue
                refined += 1
                err = abs(fd - g[c]) / max(abs(fd), 1e-30)
            errs.append(err)
        report[name] = (float(np.max(errs)), float(np.median(errs)), len(errs), refined)
    for name, (mx, med, n, refined) in report.items():
        assert n >= 32, report
        assert mx <= FD_TOL, report
    d.close()
    m.free()


def test_fp32_adjoint_tracks_fp64(gpu_lib, ctx):
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx)
    grads = {}
    for prec in (1, 0):
        d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=prec)
        target = d.forward(lnT + 0.05, lnX, b)
        flux = d.forward(lnT, lnX, b)
        gflux = 2.0 * (flux - target) / target.abs().max() ** 2
        grads[prec] = [g.cpu().numpy() for g in d.backward(gflux)]
        d.close()
    for g64, g32 in zip(grads[1], grads[0]):
        # the FP32 node values move a few SUBGRID window decisions relative to FP64: the
        # gradient as a whole agrees to 1e-2, single significant cells to 5e-2
        assert np.linalg.norm(g32 - g64) <= 1e-2 * np.linalg.norm(g64)
        sel = np.abs(g64) > 1e-2 * np.abs(g64).max()
        rel = np.abs(g32[sel] - g64[sel]) / np.abs(g64[sel])
        assert np.max(rel) <= 5e-2, np.max(rel)
    m.free()


def test_checkpoint_intervals_agree(gpu_lib, ctx):
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx)
    out = []
    for every in (1, 32):
        d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
        d.set_checkpoint(every)
        target = d.forward(lnT + 0.05, lnX, b * 0.9)
        flux = d.forward(lnT, lnX, b)
        out.append([g.cpu().numpy() for g in d.backward(2.0 * (flux - target))])
        d.close()
    for a, r in zip(*out):
        np.testing.assert_allclose(a, r, rtol=1e-12, atol=1e-12 * np.abs(r).max())
    m.free()


@pytest.mark.parametrize("name,over", [("tiny_band", {}), ("adjoint_disk", {"nphi": 4, "nlines": 3})])
@pytest.mark.parametrize("prec", [1, 0])
def test_gradient_sweep_matches_reverse_sweep(gpu_lib, ctx, name, over, prec):
    """The gradient sweep in walk order (default, interval 0: multipliers from the
    remaining optical depth) against the reverse sweep over stored intensities (interval
    1): the same gradient of the same forward. FP64: to rounding (1e-8 relative to the
    largest gradient); FP32: relative L2 difference <= 1e-3."""
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx, name, **over)
    out = []
    for every in (0, 1):
        d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=prec)
        d.set_checkpoint(every)
        target = d.forward(lnT + 0.05, lnX, b * 0.9)
        flux = d.forward(lnT, lnX, b)
        out.append([g.cpu().numpy() for g in d.backward(2.0 * (flux - target) / target.abs().max() ** 2)])
        d.close()
    for a, r in zip(*out):
        assert np.abs(r).max() > 0
        if prec == 1:
            np.testing.assert_allclose(a, r, rtol=0, atol=1e-8 * np.abs(r).max())
        else:
            assert np.linalg.norm(a - r) <= 1e-3 * np.linalg.norm(r), np.linalg.norm(a - r) / np.linalg.norm(r)
    m.free()


@pytest.mark.parametrize("prec", [1, 0])
def test_forward_keeping_optical_depths_is_the_plain_walk(gpu_lib, ctx, prec):
    """The forward of the gradient sweep (the walk that also keeps each channel's optical
    depth) renders exactly what the plain walk renders (the reverse sweep's forward)."""
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx, "adjoint_disk", nphi=4, nlines=3)
    out = []
    for every in (0, 1):
        d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=prec)
        d.set_checkpoint(every)
        out.append(d.forward(lnT, lnX, b).cpu().numpy())
        d.close()
    assert np.array_equal(out[0], out[1])
    m.free()


def test_autograd_function(gpu_lib, ctx):
    import torch
    cfg, m, lnT, lnX, b = _setup(gpu_lib, ctx)
    d = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
    target = d.forward(lnT * 1.01, lnX, b).detach()
    pT = lnT.clone().requires_grad_(True)
    pX = lnX.clone().requires_grad_(True)
    pb = b.clone().requires_grad_(True)
    flux = gpu_lib.raytrace(d, pT, pX, pb)
    loss = (((flux - target) / target.abs().max()) ** 2).sum()
    d.forward(lnT, lnX, b * 1.3)            # another forward in between: backward must not use it
    loss.backward()
    gflux = 2.0 * (d.forward(lnT, lnX, b) - target) / target.abs().max() ** 2
    gT, gX, gb = d.backward(gflux)
    # the same kernel twice: equal up to the order of the atomic accumulation per cell
    for a, r in ((pT.grad, gT), (pX.grad, gX), (pb.grad, gb)):
        r = r.cpu().numpy()
        np.testing.assert_allclose(a.cpu().numpy(), r, rtol=1e-12, atol=1e-12 * np.abs(r).max())
    d.close()
    m.free()
