"""Spectrum post-processing (pyradlite RadliteSpectrum.gen_spec, radlite.py:2420-3187).

CPU: the numpy restatement in oracle/genspec_ref.py reproduces the reference's own outputs
(tests/golden/genspec_*.json, made by running pyradlite's code) bit for bit, including the
reference's failure when the output grid overshoots the fine grid; the library's reader
of the per-core output files gives the values the reference's reader gives.

GPU: rl_gen_spec against the same fixtures and against the restatement on a larger
random band (<= 1e-12 relative: the host libm's exp and pow may differ in the last bit
between machines), and the RadliteSpectrum front end on two RADlite_gpu runs."""
import glob
import json
import os
import shutil

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "genspec_*.json")) if "reader" not in p)
KEYS = ("wavelength", "frequency", "spectrum", "emission", "continuum")


def load(path):
    with open(path) as fh:
        g = json.load(fh)
    lines = [{k: (np.array(v) if isinstance(v, list) else v) for k, v in d.items()} for d in g["lines"]]
    return g, lines


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-5] for p in CASES])
def test_restatement_reproduces_reference(path):
    from oracle import genspec_ref as G
    g, lines = load(path)
    p = g["params"]
    if "error" in g["out"]:
        assert "above the interpolation range" in g["out"]["error"]
        with pytest.raises(ValueError):
            G.process(lines, p["obsres"], p["vsampling"], p["dist"])
        return
    out = G.process(lines, p["obsres"], p["vsampling"], p["dist"])
    for k in KEYS:
        np.testing.assert_allclose(out[k], g["out"][k], rtol=1e-14, atol=0)


def test_convolve_reflect_matches_scipy():
    """The smoothing's reflected edges, as scipy.ndimage.convolve(mode='reflect') defines
    them, also for kernels longer than the grid (period 2n). gen_spec's own grids always
    make the fine grid longer than the kernel (3 obsres of box on each side)."""
    nd = pytest.importorskip("scipy.ndimage")
    from oracle import genspec_ref as G
    rng = np.random.default_rng(3)
    for n, m in ((40, 9), (40, 10), (5, 13), (7, 40), (3, 2), (4, 31), (1, 6)):
        x = rng.random(n)
        k = rng.random(m)
        k = k + k[::-1]
        np.testing.assert_allclose(G.convolve_reflect(x, k), nd.convolve(x, k, mode="reflect"), rtol=1e-13)


def test_reader_matches_reference_reader(tmp_path):
    from oracle import genspec_ref as G
    from radlite_gb300 import genspec
    with open(os.path.join(HERE, "golden", "genspec_reader.json")) as fh:
        g = json.load(fh)
    sp, mo = tmp_path / "linespectrum_moldata_0.dat", tmp_path / "moldata_0.dat"
    sp.write_text(g["spec_text"])
    mo.write_text(g["mol_text"])
    for reader in (genspec.read_core, G.read_core):
        lines, mols = reader(str(sp), str(mo))
        assert len(lines) == len(g["line"])
        for a, r in zip(lines, g["line"]):
            np.testing.assert_array_equal(a["vel"], r["vel"])
            np.testing.assert_array_equal(a["flux"], r["flux"])
            assert a["freq"] == r["freq"] and a["maxnumpoints"] == r["maxnumpoints"]
        for a, r in zip(mols, g["mol"]):
            for k in ("molname", "gup", "glow", "A", "wavenum", "freq", "Eup", "vup", "vlow", "qup", "qlow", "incl"):
                assert a[k] == r[k], k


def test_duplicate_lines_removed(tmp_path):
    """Two runs holding the same core output: every line is kept once."""
    from radlite_gb300 import genspec
    with open(os.path.join(HERE, "golden", "genspec_reader.json")) as fh:
        g = json.load(fh)
    for run in ("a", "b"):
        d = tmp_path / run
        d.mkdir()
        (d / "linespectrum_moldata_0.dat").write_text(g["spec_text"])
        (d / "moldata_0.dat").write_text(g["mol_text"])
    lines, mols = genspec.read_runs([str(tmp_path / "a"), str(tmp_path / "b")])
    assert len(lines) == len(g["line"])


# ------------------------------------------------------------------------------------
# GPU
# ------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-5] for p in CASES])
def test_gpu_matches_reference(gpu_lib, ctx, path):
    g, lines = load(path)
    p = g["params"]
    if "error" in g["out"]:
        with pytest.raises(gpu_lib.RLError, match="above the interpolation range"):
            ctx.gen_spec(lines, p["obsres"], p["vsampling"], p["dist"])
        return
    out = ctx.gen_spec(lines, p["obsres"], p["vsampling"], p["dist"])
    for k in KEYS:
        ref = np.array(g["out"][k])
        np.testing.assert_allclose(out[k], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def random_band(seed, nlines, nch):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nlines):
        vel = np.linspace(-20.0, 20.0, nch)
        flux = (1 + 0.001 * vel) * rng.uniform(1e-20, 2e-20) + rng.uniform(0, 4e-20) * np.exp(-(vel / rng.uniform(2, 6)) ** 2)
        out.append({"vel": np.array([float("%.6e" % x) for x in vel]), "flux": np.array([float("%.6e" % x) for x in flux]),
                    "freq": 2.99792458e10 * rng.uniform(2000.0, 2020.0), "maxnumpoints": nch})
    return out


@pytest.mark.gpu
def test_gpu_matches_restatement_on_a_band(ctx):
    from oracle import genspec_ref as G
    lines = random_band(11, 400, 81)
    ref = G.process(lines, 3.0, 1.0, 140.0)
    out = ctx.gen_spec(lines, 3.0, 1.0, 140.0)
    for k in KEYS:
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-12, atol=1e-12 * np.abs(ref[k]).max())


@pytest.mark.gpu
def test_radlite_spectrum_on_runs(gpu_lib, ctx, tmp_path):
    """Two model runs rendered by RADlite_gpu, laid out as pyradlite's per-core outputs,
    combined by the RadliteSpectrum front end and by the restatement."""
    from oracle import genspec_ref as G
    from radlite_gb300 import genspec, synth
    runs = []
    for i, incl in enumerate((30.0, 30.0)):
        cfg = synth.config_by_name("tiny_band", nlines=3 + i, incl_deg=incl, seed=7 + i)
        d = synth.write_model(cfg, str(tmp_path / f"m{i}"))
        gpu_lib.run_dir(d)
        run = tmp_path / f"run{i}"
        run.mkdir()
        shutil.copy(os.path.join(d, "linespectrum_moldata.dat"), run / "linespectrum_moldata_0.dat")
        shutil.copy(os.path.join(d, "moldata.dat"), run / "moldata_0.dat")
        runs.append(str(run))
    s = genspec.RadliteSpectrum({"run_paths": runs, "dist": 140.0, "obsres": 3.0, "vsampling": 1.0,
                                 "interpolation": "linear"}, ctx=ctx)
    s.gen_spec()
    lines, _ = G.read_runs(runs)
    assert len(lines) == 4          # the first run's three lines are also in the second
    ref = G.process(lines, 3.0, 1.0, 140.0)
    for k in KEYS:
        np.testing.assert_allclose(s.get_attr(k), ref[k], rtol=1e-12, atol=1e-12 * np.abs(ref[k]).max())
    assert s.get_unit("spectrum") == "Jy"
