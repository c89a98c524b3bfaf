"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Tolerances: FP32 transfer (FP64 geometry) <= 1e-4 relative in every channel whose flux
exceeds 1e-3 of the line peak; FP64 transfer <= 1e-9 relative (same algorithm, same
inputs, different summation order and math library)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
FP64_TOL = 1e-9


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", ["tiny_line", "tiny_band", "small_line"])
def test_spectra_fp32_and_fp64(ctx, oracle_lib, model_dir, name):
    d = model_dir(name)
    o = oracle_lib.Oracle(d)
    m = ctx.load_dir(d)
    lines = list(range(o.ilinestart, o.ilinestart + o.nlines_spec))
    refs = [o.line_spectrum(il) for il in lines]
    for il, (ref, rvelo, rcnt) in zip(lines, refs):
        got, velo, st = m.calc_line_spectrum(il, stats=True)
        np.testing.assert_allclose(velo, rvelo, rtol=0, atol=1e-9)
        assert relerr(got, ref) <= FP32_TOL, (name, il, relerr(got, ref))
    m.set_precision(1)
    for il, (ref, _, rcnt) in zip(lines, refs):
        got, _, st = m.calc_line_spectrum(il, stats=True)
        assert relerr(got, ref) <= FP64_TOL, (name, il, relerr(got, ref))
        # same channel selection and sub-stepping decisions as the oracle
        assert st["integrated"] == rcnt["integrated"]
        assert abs(st["steps"] - rcnt["steps"]) <= 1e-6 * rcnt["steps"] + 2
    m.free()


def test_multi_line_launch_matches_single(ctx, model_dir):
    d = model_dir("tiny_band")
    m = ctx.load_dir(d)
    info = m.info()
    many = m.spectra(info["ilinestart"], info["nlines_spec"])
    for k in range(info["nlines_spec"]):
        one, _ = m.calc_line_spectrum(info["ilinestart"] + k)
        np.testing.assert_allclose(many[k], one, rtol=1e-12)
    m.free()


def test_image_fp64_matches_oracle(ctx, oracle_lib, model_dir):
    d = model_dir("tiny_line")
    o = oracle_lib.Oracle(d)
    m = ctx.load_dir(d)
    m.set_precision(1)
    img = m.line_image(o.ilinestart)
    ref, mask, _ = o.line_image(o.ilinestart)
    scale = np.abs(ref).max()
    assert np.max(np.abs(img - ref)) <= 1e-9 * scale
    m.set_precision(0)
    img32 = m.line_image(o.ilinestart)
    assert np.max(np.abs(img32 - ref)) <= 2e-4 * scale
    m.free()


@pytest.mark.parametrize("name,incl", [("tiny_line", 45.0), ("tiny_line", 5.0), ("tiny_band", 85.0)])
def test_trajectories_match_oracle(ctx, oracle_lib, model_dir, name, incl):
    d = model_dir(name, incl_deg=incl)
    o = oracle_lib.Oracle(d)
    m = ctx.load_dir(d)
    for ray in list(range(0, o.nrays, max(1, o.nrays // 60))) + [o.nrays - 1]:
        a = o.trajectory(ray)
        b = m.trajectory(ray)
        assert len(a["s"]) == len(b["s"])
        for k in ("icr", "ir", "it"):
            np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_allclose(b["s"], a["s"], rtol=0, atol=1e-12 * np.abs(a["s"]).max())
        np.testing.assert_allclose(b["mu"], a["mu"], rtol=0, atol=1e-12)
    m.free()


def test_run_dir_output_file(gpu_lib, oracle_lib, model_dir, tmp_path):
    import shutil
    src = model_dir("tiny_band")
    a, b = str(tmp_path / "gpu"), str(tmp_path / "cpu")
    shutil.copytree(src, a)
    shutil.copytree(src, b)
    gpu_lib.run_dir(a)
    oracle_lib.run_dir(b)
    fa = os.path.join(a, "linespectrum_moldata.dat")
    fb = os.path.join(b, "linespectrum_moldata.dat")
    assert os.path.exists(os.path.join(a, "radlite.success"))
    la, lb = open(fa).read().split("\n"), open(fb).read().split("\n")
    assert la[:7] == lb[:7]
    sa, sb = gpu_lib.read_spectrum_file(fa), gpu_lib.read_spectrum_file(fb)
    assert len(sa) == len(sb) == 6
    for x, y in zip(sa, sb):
        assert (x["up"], x["low"]) == (y["up"], y["low"])
        np.testing.assert_array_equal(x["velo"], y["velo"])
        assert relerr(x["flux"], y["flux"]) <= FP32_TOL + 5e-7


def test_executable(gpu_lib, model_dir, tmp_path):
    import shutil
    import subprocess
    d = str(tmp_path / "m")
    shutil.copytree(model_dir("tiny_line"), d)
    r = subprocess.run([gpu_lib.EXE_PATH, d], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(os.path.join(d, "linespectrum_moldata.dat"))
    log = open(os.path.join(d, "radlite.log")).read()
    assert "RUN OF RADICAL" in log and "Finishing Date" in log and "END OF RUN RADLITE" in log
    # a SAVE_IMCIR build's circular images beside the spectrum
    r = subprocess.run([gpu_lib.EXE_PATH, "--save-imcir", d], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(os.path.join(d, "lineposvelcirc_moldata_1.dat"))
    assert open(os.path.join(d, "radlite.log")).read().count("RUN OF RADICAL") == 2
    os.remove(os.path.join(d, "density.inp"))
    r = subprocess.run([gpu_lib.EXE_PATH, d], capture_output=True, text=True)
    assert r.returncode == 13 and "density.inp" in r.stderr


def test_executable_posvel_and_manifest(gpu_lib, tmp_path):
    """linespectrum.inp command 2 through the executable; a manifest of such directories
    is refused (a batch renders line spectra)."""
    import subprocess
    from radlite_gb300 import synth
    d = synth.write_model(synth.config_by_name("tiny_line", command=2, pv_nx=6, pv_ny=4, nlines=2, ilinestart=1),
                          str(tmp_path / "pv"))
    r = subprocess.run([gpu_lib.EXE_PATH, d], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for il in (1, 2):
        f = gpu_lib.read_posvel_file(os.path.join(d, f"lineposvel_moldata_{il}.dat"))
        assert f["temp"].shape == (f["nfr"], 4, 6) and f["temp"].max() > 0
    assert not os.path.exists(os.path.join(d, "linespectrum_moldata.dat"))
    man = tmp_path / "models.txt"
    man.write_text(d + "\n")
    r = subprocess.run([gpu_lib.EXE_PATH, "--manifest", str(man)], capture_output=True, text=True)
    assert r.returncode == 13 and "command 0" in r.stderr


def test_arrays_path_matches_files(ctx, model_dir):
    from radlite_gb300 import synth
    cfg = synth.config_by_name("tiny_band")
    m1 = ctx.load_dir(model_dir("tiny_band"))
    arr = synth.model_arrays(cfg)
    cam = dict(incl_deg=cfg.incl_deg, nphi=cfg.nphi, dbdr=cfg.dbdr, nrrayextra=cfg.nrrextra, vmax=cfg.vmax,
               dv=cfg.dv, ilinestart=cfg.ilinestart, nlines=cfg.nlines)
    m2 = ctx.load_arrays(arr, cam)
    f1 = m1.spectra(1, cfg.nlines)
    f2 = m2.spectra(1, cfg.nlines)
    for k in range(cfg.nlines):
        assert relerr(f2[k], f1[k]) <= 1e-5
    m1.free()
    m2.free()
