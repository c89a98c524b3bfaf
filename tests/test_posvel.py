"""Position-velocity cube (linespectrum.inp command 2; telescope.F:1828-2475).

CPU: the oracle's rectangular camera and cube (every pixel is the all-channel spectrum of
its ray without star mixing; pixels outside 0.999 R_nr are empty; the unresolved star is
smeared over the four central pixels), its optical depth against an independent
trapezoid of the dust opacity, and the host reader of the command-2 request.

GPU: the CUDA cube against the oracle's (FP64 <= 1e-10 relative, FP32 <= 1e-4 relative on
values above 1e-3 of the peak, the tolerance of the line spectra), with and without the
star, rotated and offset; RADlite_gpu's lineposvel files against the API cube."""
import math
import os

import numpy as np
import pytest

from radlite_gb300 import synth


def pv_cfg(**over):
    base = dict(command=2, pv_nx=8, pv_ny=6, nlines=2, ilinestart=1)
    base.update(over)
    return synth.config_by_name("tiny_line", **base)


def test_oracle_cube_assembles_ray_spectra(oracle_lib, tmp_path):
    d = synth.write_model(pv_cfg(pv_size_au=0.0), str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    assert o.command == 2 and o.ilinestart == 1
    pv = o.pv
    I, tau = o.posvel(1, **pv)
    x0, z0, b, (unres, spx, spy, srat, theta0) = o.pv_rays(**pv)
    nx, ny = pv["nx"], pv["ny"]
    assert unres == 1 and 0.0 < srat < 1.0
    rmax = np.loadtxt(os.path.join(d, "radius.inp"), skiprows=1)[-1]
    star_I, _ = o.ray_spectrum(1, 0.0, 0.0)
    empty = 0
    for ix in range(nx):
        for iy in range(ny):
            r = ix * ny + iy
            central = ix in (nx // 2 - 1, nx // 2) and iy in (ny // 2 - 1, ny // 2)
            if b[r] >= 0.999 * rmax:
                ref_I, ref_t = np.zeros(o.nfr), np.zeros(o.nfr)
                empty += 1
            else:
                ref_I, ref_t = o.ray_spectrum(1, x0[r], z0[r])
            if central:
                ref_I = star_I * srat + (1.0 - srat) * ref_I
            np.testing.assert_array_equal(I[:, iy, ix], ref_I)
            np.testing.assert_array_equal(tau[:, iy, ix], ref_t)
    assert empty > 0                       # the image corners lie outside the grid
    assert tau.max() > 1.0                 # the line is optically thick somewhere


def test_oracle_tau_thin_dust_trapezoid(oracle_lib, tmp_path):
    """Without line opacity, char_tau of every channel is the trapezoid sum of the dust
    extinction over the ray's segments (central-hole segments have zero length)."""
    cfg = synth.config_by_name("tiny_line", abund=0.0, nphi=8)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    x0, z0, _, _ = o.rays()
    r = np.loadtxt(os.path.join(d, "radius.inp"), skiprows=1)
    th = np.loadtxt(os.path.join(d, "theta.inp"), skiprows=1)
    drho = np.loadtxt(os.path.join(d, "dustdens.inp"), skiprows=1).reshape(cfg.nr, cfg.nt)
    acell = drho * cfg.kappa_abs

    def a_at(rr, tt):
        tt = min(tt, np.pi - tt)
        ri = np.interp(rr, r, np.arange(cfg.nr))
        ti = np.interp(tt, th, np.arange(cfg.nt))
        i0, j0 = int(ri), int(ti)
        i1, j1 = min(i0 + 1, cfg.nr - 1), min(j0 + 1, cfg.nt - 1)
        a, bb = ri - i0, ti - j0
        return (1 - a) * ((1 - bb) * acell[i0, j0] + bb * acell[i0, j1]) + a * ((1 - bb) * acell[i1, j0] + bb * acell[i1, j1])

    for ray in (1 + 8 * 3, 1 + 8 * 20 + 5):
        _, tau = o.ray_spectrum(cfg.ilinestart, x0[ray], z0[ray])
        t = o.trajectory(ray)
        al = np.array([a_at(rr, tt) for rr, tt in zip(t["r"], t["theta"])])
        ds = np.diff(t["s"])
        hole = (t["ir"][1:] == 1) & (t["ir"][:-1] == 1) & (t["icr"][1:] == 1) & (t["icr"][:-1] == 1)
        ds[hole] = 0.0
        expect = np.sum(0.5 * (al[1:] + al[:-1]) * ds)
        assert expect > 0
        np.testing.assert_allclose(tau, expect, rtol=1e-9)


def test_host_reads_posvel_request(gpu_lib, tmp_path):
    cfg = pv_cfg(pv_nx=10, pv_ny=4, pv_phioff=0.3, pv_xoff_au=0.5, pv_yoff_au=-0.25, pv_addstar=0, ilinestart=2)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    m = gpu_lib.load_dir_host(d)
    sp = m.posvel_spec()
    assert (sp["nx"], sp["ny"], sp["addstar"]) == (10, 4, 0)
    assert sp["phioff"] == pytest.approx(0.3) and sp["xoff"] == pytest.approx(0.5 * synth.AU, rel=1e-9)
    assert m.info()["ilinestart"] == 1     # main.F:204: the run starts at line 1
    with pytest.raises(gpu_lib.RLError, match="even"):
        m.set_posvel(7, 4, 1e15, 1e15)
    with pytest.raises(gpu_lib.RLError, match="star-centred"):
        m.set_posvel(8, 4, 1e15, 1e15, xoff=1e13, addstar=1)
    m.set_posvel(8, 4, 2e15, 1e15, addstar=1)
    assert m.posvel_spec()["nx"] == 8


def test_arcsec_size_specifier_reads_as_cm(gpu_lib, oracle_lib, tmp_path):
    """Size specifier 0 (arcsec): the reference warns and reads the sizes as for 1
    (telescope.F:207-216), so both readers take the same request."""
    d1 = synth.write_model(pv_cfg(), str(tmp_path / "cm"))
    d0 = synth.write_model(pv_cfg(), str(tmp_path / "as"))
    p = tmp_path / "as" / "linespectrum.inp"
    txt = p.read_text()
    assert "1       image size in cm?" in txt
    p.write_text(txt.replace("1       image size in cm?", "0       image size in cm?"))
    m1, m0 = gpu_lib.load_dir_host(d1), gpu_lib.load_dir_host(d0)
    assert m0.posvel_spec() == m1.posvel_spec()
    assert oracle_lib.Oracle(d0).pv == oracle_lib.Oracle(d1).pv
    p.write_text(txt.replace("1       image size in cm?", "2       image size in cm?"))
    with pytest.raises(gpu_lib.RLError, match="size specifier"):
        gpu_lib.load_dir_host(d0)


# ------------------------------------------------------------------------------------
# GPU
# ------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _cmp(got, ref, tol):
    sel = np.abs(ref) > 1e-3 * np.abs(ref).max()
    err = np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])
    assert err.max() <= tol, (err.max(), tol)
    # values below the cut agree in absolute terms at the cut's scale
    assert np.abs(got - ref).max() <= max(tol, 1e-6) * np.abs(ref).max()


CASES = {
    "star": dict(),
    "rotated_offset": dict(pv_phioff=0.4, pv_xoff_au=0.3, pv_yoff_au=-0.2, pv_addstar=0, pv_nx=10, pv_ny=8),
    "resolved_star": dict(pv_size_au=0.0015, pv_nx=6, pv_ny=6, incl_deg=80.0),
    # the rectangular camera raises every inclination below 0.1 rad to 0.1, negative
    # ones included (telescope.F:2289-2300)
    "low_incl": dict(incl_deg=3.0, pv_nx=6, pv_ny=6),
    "negative_incl": dict(incl_deg=-30.0, pv_nx=6, pv_ny=6, pv_addstar=0),
    "cmb_boundary": dict(outer_bc=2, pv_nx=8, pv_ny=4),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_cube_matches_oracle(gpu_lib, oracle_lib, ctx, tmp_path, case):
    cfg = pv_cfg(**CASES[case])
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    m = ctx.load_dir(d)
    sp = m.posvel_spec()
    refs = [o.posvel(il, **o.pv) for il in (1, 2)]
    m.set_precision(1)
    I, tau, st = m.posvel(1, 2, stats=True)
    assert st["nlines"] == 2 and st["ray_channels"] > 0
    for k, (rI, rt) in enumerate(refs):
        assert I[k].shape == (o.nfr, sp["ny"], sp["nx"])
        _cmp(I[k], rI, 1e-10)
        _cmp(tau[k], rt, 1e-10)
    m.set_precision(0)
    I32, tau32 = m.posvel(1, 2)
    for k, (rI, rt) in enumerate(refs):
        _cmp(I32[k], rI, 1e-4)
        _cmp(tau32[k], rt, 1e-4)
    m.free()


@pytest.mark.gpu
def test_gpu_cube_outside_the_grid(gpu_lib, oracle_lib, ctx, tmp_path):
    """An image offset beyond the outer radius traces no ray: every pixel is empty
    (telescope.F:2136-2146), in both precisions."""
    cfg = pv_cfg(pv_xoff_au=1.0e4, pv_addstar=0, pv_nx=4, pv_ny=4)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    I_ref, tau_ref = oracle_lib.Oracle(d).posvel(1, **oracle_lib.Oracle(d).pv)
    assert not I_ref.any() and not tau_ref.any()
    m = ctx.load_dir(d)
    for prec in (0, 1):
        m.set_precision(prec)
        I, tau, st = m.posvel(1, 1, stats=True)
        assert st["nrays"] == 0 and not I.any() and not tau.any()
    m.free()


@pytest.mark.gpu
def test_run_dir_writes_posvel_files(gpu_lib, ctx, tmp_path):
    cfg = pv_cfg(ilinestart=2)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    gpu_lib.run_dir(d)
    assert os.path.exists(os.path.join(d, "radlite.success"))
    m = ctx.load_dir(d)
    info = m.info()
    I, tau = m.posvel(1, cfg.nlines)
    for k in range(cfg.nlines):
        f = gpu_lib.read_posvel_file(os.path.join(d, f"lineposvel_moldata_{k + 1}.dat"))
        assert (f["nx"], f["ny"], f["nfr"]) == (cfg.pv_nx, cfg.pv_ny, info["nfr"])
        assert f["incl_deg"] == pytest.approx(cfg.incl_deg, abs=1e-3) and f["distance_pc"] == 1.0
        temp = 3.25465503368e36 / f["freq"] ** 2 * I[k]
        np.testing.assert_allclose(f["temp"], temp, rtol=6e-5, atol=1e-6 * np.abs(temp).max())
        np.testing.assert_allclose(f["tau"], tau[k], rtol=6e-5, atol=1e-6 * np.abs(tau[k]).max())
        v = f["velo"]
        assert v[0] > 0 > v[-1] and abs(v[0] + v[-1]) < 1e-3 * abs(v[0])
    m.free()
