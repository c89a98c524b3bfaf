"""Known-answer tests that pin the CPU oracle (the reference ships no golden vectors)."""
import math
import os

import numpy as np
import pytest

from radlite_gb300 import synth


def test_keplerian_line_symmetric(oracle_lib, model_dir):
    """A Keplerian disk line is symmetric in velocity (azimuth phi <-> -phi)."""
    o = oracle_lib.Oracle(model_dir("tiny_line"))
    for iline in (1, 2, 3):
        flux, velo, cnt = o.line_spectrum(iline)
        assert np.all(np.isfinite(flux)) and flux.max() > 0
        # to 1e-6 of the peak: the window and sub-step decisions are taken in FP32 / on
        # discrete thresholds, which breaks the mirror symmetry in the far wings
        np.testing.assert_allclose(flux, flux[::-1], rtol=0, atol=1e-6 * flux.max())
        np.testing.assert_allclose(velo, -velo[::-1], atol=1e-9)
        assert cnt["steps"] > cnt["integrated"] > 0


def test_star_only_central_beam(oracle_lib, tmp_path):
    """No gas opacity, no dust: only the central beam sees the star, F = pi R*^2 I*/d^2."""
    cfg = synth.config_by_name("tiny_line", abund=0.0, kappa_abs=0.0)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    flux, _, _ = o.line_spectrum(cfg.ilinestart)
    f = synth.make_fields(cfg)
    # moldata.dat stores energies with 4 decimals (F12.4): the line frequency follows them
    nu0 = synth.line_freqs(cfg, np.round(f["E"], 4), f["lines"])[cfg.ilinestart - 1]
    fr = synth.dust_frequency_grid(cfg, f["E"], f["lines"])
    rstar = cfg.rstar_rsun * synth.RSUN
    # the reference interpolates the stellar intensity linearly on frequency.inp
    fstar = math.pi * synth.planck(fr, cfg.tstar) * rstar ** 2 / synth.PC ** 2
    nfr = o.nfr
    P = 3.33567e-6 * nu0 * o.vmax
    fq = nu0 + (-P + np.arange(nfr) * (2 * P / (nfr - 1)))
    istar = np.interp(fq, fr, 3.0308410e36 * np.array([float("%.7e" % x) for x in fstar]) / float("%.7e" % rstar) ** 2)
    expect = math.pi * float("%.7e" % rstar) ** 2 * istar / (3.08572e18 ** 2)
    np.testing.assert_allclose(flux, expect, rtol=1e-6)


def test_dust_only_continuum_flat(oracle_lib, tmp_path):
    """Without line opacity every channel of every ray carries the same continuum."""
    cfg = synth.config_by_name("tiny_line", abund=0.0)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    img, mask, _ = o.line_image(cfg.ilinestart)
    assert np.all(img > 0)
    # (the central beam, row 0, carries the frequency-dependent stellar intensity)
    np.testing.assert_allclose(img[1:], img[1:, :1].repeat(img.shape[1], 1), rtol=1e-12)
    # only the first channel is integrated (all rays but the central one copy it)
    assert mask[1:, 1:].sum() == 0 and mask[0].all()


def test_optically_thick_saturates_to_planck(oracle_lib, tmp_path):
    """Isothermal, static, very dense: line-centre intensity saturates at B_nu(T)."""
    T = 300.0
    # a vertically thick, dense envelope over nearly the whole sphere: every ray that
    # passes well inside the outer radius is optically thick in the line and the dust
    cfg = synth.config_by_name("tiny_line", t0=T, t_pow=0.0, sigma0=1e7, h0=1.0, h_pow=0.0, theta_open=1.5,
                               mstar=1e-12, nphi=8, vmax=3.0, dv=0.5, incl_deg=60.0)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    img, _, _ = o.line_image(cfg.ilinestart, 1 + 8 * 20, 1 + 8 * 40)
    f = synth.make_fields(cfg)
    nu0 = synth.line_freqs(cfg, np.round(f["E"], 4), f["lines"])[cfg.ilinestart - 1]
    B = 1.47455e-47 * nu0 ** 3 / math.expm1(4.7989e-11 * nu0 / T)
    kc = o.nfr // 2
    np.testing.assert_allclose(img[:, kc], B, rtol=2e-3)


def test_thin_dust_trapezoid(oracle_lib, tmp_path):
    """Optically thin dust (tau per segment < 1e-9): I = sum of trapezoids of j over ds."""
    cfg = synth.config_by_name("tiny_line", abund=0.0, kappa_abs=1e-12, nphi=8)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    ray = 1 + 8 * 20
    img, _, _ = o.line_image(cfg.ilinestart, ray, ray + 1)
    t = o.trajectory(ray)
    f = synth.make_fields(cfg)
    nu0 = synth.line_freqs(cfg, np.round(f["E"], 4), f["lines"])[cfg.ilinestart - 1]
    # independent interpolation of the dust emissivity at the nodes (ir, it already mirrored)
    r = np.loadtxt(os.path.join(d, "radius.inp"), skiprows=1)
    th = np.loadtxt(os.path.join(d, "theta.inp"), skiprows=1)
    drho = np.loadtxt(os.path.join(d, "dustdens.inp"), skiprows=1).reshape(cfg.nr, cfg.nt)
    temp = np.loadtxt(os.path.join(d, "dusttemp_final.dat"), skiprows=3).reshape(cfg.nr, cfg.nt)
    kap = 1e-12
    jcell = drho * kap * (1.47455e-47 * nu0 ** 3 / np.expm1(4.7989e-11 * nu0 / temp) + 1e-290)
    thfull = np.concatenate([th, np.pi - th[::-1]])
    def j_at(rr, tt):
        tt = min(tt, np.pi - tt)           # mirror
        ri = np.interp(rr, r, np.arange(cfg.nr))
        ti = np.interp(tt, th, np.arange(cfg.nt))
        i0, j0 = int(ri), int(ti)
        i1, j1 = min(i0 + 1, cfg.nr - 1), min(j0 + 1, cfg.nt - 1)
        a, b = ri - i0, ti - j0
        return (1 - a) * ((1 - b) * jcell[i0, j0] + b * jcell[i0, j1]) + a * ((1 - b) * jcell[i1, j0] + b * jcell[i1, j1])
    js = np.array([j_at(rr, tt) for rr, tt in zip(t["r"], t["theta"])])
    ds = np.diff(t["s"])
    hole = (t["ir"][1:] == 1) & (t["ir"][:-1] == 1) & (t["icr"][1:] == 1) & (t["icr"][:-1] == 1)
    ds[hole] = 0.0
    expect = np.sum(0.5 * (js[1:] + js[:-1]) * ds)
    np.testing.assert_allclose(img[0, 0], expect, rtol=1e-3)


def test_geometry_properties(oracle_lib, model_dir):
    """s strictly increasing with the eps*r separation, radii inside the grid."""
    o = oracle_lib.Oracle(model_dir("small_line"))
    r = np.loadtxt(os.path.join(model_dir("small_line"), "radius.inp"), skiprows=1)
    for ray in range(0, o.nrays, 97):
        t = o.trajectory(ray)
        assert len(t["s"]) >= 2
        assert np.all(np.diff(t["s"]) > 1e-10 * t["r"][1:] * 0.999)
        assert np.all(t["r"] <= r[-1] * (1 + 1e-9)) and np.all(t["r"] >= r[0] * (1 - 1e-9))
        assert np.all((t["icr"] >= 1) & (t["icr"] <= 3))
        assert np.all(np.abs(t["mu"]) <= 1.0)


def test_isothermal_lte_slab_law(oracle_lib, tmp_path):
    """One gas temperature everywhere, LTE populations, no dust: the source function
    j/alpha is the same at every node and every SUBGRID point (the interpolation keeps the
    population ratio), and the linear-source step gives q = (1 - x) S exactly, which the
    bracket at the theoretical maximum never clips (1 - e^-dtau <= dtau). Every ray and
    channel then satisfies I = S (1 - e^-tau) with its own char_tau, however the walk
    sub-steps, and S is the Planck function at the line frequency and that temperature
    (to the 1e-5 of the physical constants' variants)."""
    cfg = synth.config_by_name("tiny_line", t_pow=0.0, kappa_abs=0.0, nlines=1)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    x0, z0, _, _ = o.rays()
    ratios, thick = [], 0
    for k in range(0, len(x0), 23):
        I, tau = o.ray_spectrum(cfg.ilinestart, x0[k], z0[k])
        sel = tau > 1e-4
        ratios.append(I[sel] / -np.expm1(-tau[sel]))
        thick += int(np.sum(tau > 3.0))
    r = np.concatenate(ratios)
    assert r.size > 100 and thick > 0          # thin and thick channels both present
    S = float(np.mean(r))
    assert np.max(np.abs(r / S - 1.0)) <= 1e-7
    f = synth.make_fields(cfg)
    u, l, _ = f["lines"][cfg.ilinestart - 1]
    E = np.round(f["E"], 4)                      # moldata.dat's F12.4 energies
    nu = (E[u - 1] - E[l - 1]) * 2.99792458e10
    h, kb, c = 6.62607015e-27, 1.380649e-16, 2.99792458e10
    B = 2.0 * h * nu ** 3 / c ** 2 / math.expm1(h * nu / (kb * cfg.t0))
    assert abs(S / B - 1.0) <= 1e-4
