"""The masing test of charintline (telescope.F:4291-4297): a segment whose line opacity at
its end times its length falls below -0.01 sets maserflag, and the reference prints
"WARNING: Masing detected!" after the line (telescope.F:1649-1652, 2020-2023). The models
here carry a population inversion in one radial shell (upper level set to k times the
lower one's statistical share), written into the level populations file.

CPU: the oracle flags it for inversions that reach the threshold and not for one far below
it or for the plain model. GPU: the library's flags equal the oracle's for spectra (FP32
and FP64), the circular image and the position-velocity cube; FP64 spectra keep 1e-9,
FP32 spectra 1e-4 (1e-3 where masing amplifies the intensity); RADlite_gpu prints the
reference's warning."""
import os

import numpy as np
import pytest

from radlite_gb300 import synth


def inverted_model(tmp_path, tag, k, shell, iline=None, **over):
    cfg = synth.config_by_name("tiny_line", **over)
    d = synth.write_model(cfg, str(tmp_path / tag))
    if k is None:
        return cfg, d
    E, g, lines = synth.molecule_levels(cfg)
    up, lo, _ = lines[(iline or cfg.ilinestart) - 1]
    p = os.path.join(d, "levelpop_moldata.dat")
    rows = open(p).read().split("\n")
    head, body = rows[:3], [r for r in rows[3:] if r.strip()]
    out = []
    for c, r in enumerate(body):
        v = [float(x) for x in r.split("\t")]
        if c // cfg.nt + 1 == shell:
            v[up - 1] = k * v[lo - 1] * g[up - 1] / g[lo - 1]
        out.append("\t".join("%.10e" % x for x in v))
    open(p, "w").write("\n".join(head + out) + "\n")
    return cfg, d


CASES = [("plain", None, 0, False), ("mild", 1.0002, 12, True), ("outer", 1.001, 22, True),
         ("below", 1.0 + 1e-9, 22, False)]


@pytest.mark.parametrize("tag,k,shell,flag", CASES, ids=[c[0] for c in CASES])
def test_oracle_flags_masing(oracle_lib, tmp_path, tag, k, shell, flag):
    cfg, d = inverted_model(tmp_path, tag, k, shell)
    o = oracle_lib.Oracle(d)
    o.line_spectrum(cfg.ilinestart)
    assert o.masing() == flag


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


@pytest.mark.gpu
@pytest.mark.parametrize("tag,k,shell,flag", CASES, ids=[c[0] for c in CASES])
def test_gpu_flags_match_oracle(gpu_lib, oracle_lib, tmp_path, tag, k, shell, flag):
    cfg, d = inverted_model(tmp_path, tag, k, shell)
    o = oracle_lib.Oracle(d)
    ref, _, cnt = o.line_spectrum(cfg.ilinestart)
    assert o.masing() == flag
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    got, _ = m.calc_line_spectrum(cfg.ilinestart)
    assert m.masing(cfg.ilinestart) == flag
    # a masing segment multiplies the intensity by e^|tau| and the FP32 rounding of its
    # negative optical depth with it: FP32 holds 1e-3 there, 1e-4 elsewhere
    assert relerr(got, ref) <= (1e-3 if flag else 1e-4)
    m.set_precision(1)
    got, _, st = m.calc_line_spectrum(cfg.ilinestart, stats=True)
    assert m.masing(cfg.ilinestart) == flag
    assert relerr(got, ref) <= 1e-9 and st["integrated"] == cnt["integrated"]
    m.line_image(cfg.ilinestart)
    assert m.masing(cfg.ilinestart) == flag
    # the position-velocity cube of the same line over the disk
    size = 2.0 * float(synth.make_grid(cfg)[0][-1])
    m.set_posvel(8, 8, size, size, addstar=1)
    m.posvel(cfg.ilinestart, 1)
    o.posvel(cfg.ilinestart, 8, 8, size, size, addstar=1)
    assert m.masing(cfg.ilinestart) == o.masing()
    m.free()
    ctx.close()


@pytest.mark.gpu
def test_run_dir_prints_the_warning(gpu_lib, tmp_path, capfd):
    # a directory run renders lines 1.. (main.F:204): invert line 1
    cfg, d = inverted_model(tmp_path, "run", 1.001, 20, iline=1)
    gpu_lib.run_dir(d)
    out = capfd.readouterr().out
    assert "          WARNING: Masing detected!\n Will only warn once for this transition.\n" in out
    _, d0 = inverted_model(tmp_path, "run0", None, 0)
    gpu_lib.run_dir(d0)
    assert "Masing" not in capfd.readouterr().out


def test_masing_query_arguments(gpu_lib, tmp_path):
    """Host only: before any render no line is flagged; bad line indices are errors."""
    cfg, d = inverted_model(tmp_path, "m", 1.001, 22)
    m = gpu_lib.load_dir_host(d)
    assert m.masing(cfg.ilinestart) is False
    for bad in (0, 10 ** 6):
        with pytest.raises(gpu_lib.RLError, match="line index"):
            m.masing(bad)
    m.free()


@pytest.mark.gpu
def test_batch_flags_match_oracle(gpu_lib, oracle_lib, tmp_path, capfd):
    """A batch of the four models: each job's flag equals the oracle's, spectra as the
    per-model renders; a manifest run prints the warning for the inverted directories."""
    ctx = gpu_lib.Context(0)
    models, want, dirs = [], [], []
    b = gpu_lib.Batch(ctx)
    for tag, k, shell, flag in CASES:
        cfg, d = inverted_model(tmp_path, "b" + tag, k, shell)
        o = oracle_lib.Oracle(d)
        o.line_spectrum(cfg.ilinestart)
        assert o.masing() == flag
        m = ctx.load_dir(d)
        models.append(m)
        want.append(flag)
        dirs.append(d)
        b.add(m, cfg.ilinestart, 1)
    for run in range(2):   # the first run and a graph replay
        b.run()
        for j, flag in enumerate(want):
            assert list(b.masing(j)) == [flag], (run, j)
    b.close()
    for m in models:
        m.free()
    ctx.close()
    man = tmp_path / "models.txt"
    # a directory run renders lines 1.. (main.F:204): invert line 1 of one directory
    _, dinv = inverted_model(tmp_path, "man_inv", 1.001, 20, iline=1)
    _, dplain = inverted_model(tmp_path, "man_plain", None, 0)
    man.write_text(dplain + "\n" + dinv + "\n")
    capfd.readouterr()
    gpu_lib.run_manifest(str(man))
    out = capfd.readouterr().out
    assert out.count("          WARNING: Masing detected!\n Will only warn once for this transition.\n") == 1


def test_differentiable_path_has_no_inversion(oracle_lib, tmp_path):
    """The differentiable path renders LTE populations, whose line opacity
    C (N_low B_lu - N_up B_ul) = C N_low (g_u/g_l) B_ul (1 - e^{-h nu/kT}) is positive at every
    T > 0, so the masing test cannot trigger there: the populations it derives hold
    N_up g_l <= N_low g_u in every cell, and the oracle finds no masing on that model."""
    cfg = synth.config_by_name("tiny_band")
    arr = synth.lte_arrays(cfg)
    _, g, lines = synth.molecule_levels(cfg)
    pop = arr["pop"]
    for up, lo, _ in lines[cfg.ilinestart - 1:cfg.ilinestart - 1 + cfg.nlines]:
        assert np.all(pop[up - 1] * g[lo - 1] <= pop[lo - 1] * g[up - 1])
    d = synth.write_model(cfg, str(tmp_path / "lte"))
    o = oracle_lib.Oracle(d)
    for k in range(cfg.nlines):
        o.line_spectrum(cfg.ilinestart + k)
        assert not o.masing()
