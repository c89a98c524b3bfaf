"""The overshoot test of qdr_src_2 (transfer.F:1548-1553, compiled into the reference's
default build): a formal-solution step whose quadrature, before the bracket at the
theoretical maximum, exceeds twice that maximum is counted in transerr_overshoot, and the
run's log warns (main.F:1547-1552); a rectangular image clears the counter before it is
made (telescope.F:2094) and prints its own warning after it (telescope.F:2204-2213).

CPU: the oracle counts such steps on the band model (steep opacity and source-function
changes across a cell at the line-window edges) and none on the single-line model; the
per-line counts are stable between calls.

GPU: with RL_CHECK_OVERSHOOT the library renders bit for bit the spectra it renders
without the check and reports 0 without it. The FP64 walk counts what the oracle counts
(measured equal on every line; the bound allows 1e-4 relative + 4 steps for a quadrature
within rounding of twice the maximum). The FP32 walk takes the test on its own steps,
which are not the FP64 ones (on this model 7.8e6 steps per line against the oracle's
8.7e6): it counts 0.9% fewer, within 2%. Position-velocity cubes always count; RADlite_gpu's
radlite.log carries the reference's start record, the overshoot warning for the band model
and none for the single-line model (largest quadrature there 1.1 times the maximum)."""
import os
import shutil

import numpy as np
import pytest

from radlite_gb300 import synth


def _model(tmp_path, name, **over):
    cfg = synth.config_by_name(name, **over)
    return cfg, synth.write_model(cfg, str(tmp_path / name))


def _oracle_counts(oracle_lib, d, cfg):
    o = oracle_lib.Oracle(d)
    out = []
    for il in range(cfg.ilinestart, cfg.ilinestart + cfg.nlines):
        o.line_spectrum(il)
        out.append(o.overshoots())
    return out


def test_oracle_counts_overshoots(oracle_lib, tmp_path):
    cfg, d = _model(tmp_path, "tiny_band")
    band = _oracle_counts(oracle_lib, d, cfg)
    assert all(c > 0 for c in band), band
    assert band == _oracle_counts(oracle_lib, d, cfg)
    cfg, d = _model(tmp_path, "tiny_line")
    assert _oracle_counts(oracle_lib, d, cfg) == [0] * cfg.nlines


def _close(got, ref, rel, slack):
    return abs(got - ref) <= rel * ref + slack


@pytest.mark.gpu
@pytest.mark.parametrize("prec,rel,slack", [(1, 1e-4, 4), (0, 2e-2, 16)])
def test_gpu_counts_match_oracle(gpu_lib, oracle_lib, tmp_path, prec, rel, slack):
    cfg, d = _model(tmp_path, "tiny_band")
    ref = _oracle_counts(oracle_lib, d, cfg)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    m.set_precision(prec)
    lines = range(cfg.ilinestart, cfg.ilinestart + cfg.nlines)
    plain, st0 = m.spectra(cfg.ilinestart, cfg.nlines, stats=True)
    assert st0["overshoots"] == 0
    per_line = [m.spectra(il, 1)[0] for il in lines]
    m.set_checks(True)
    got = []
    for k, il in enumerate(lines):
        f, st = m.spectra(il, 1, stats=True)
        assert np.array_equal(f[0], per_line[k]), il
        got.append(st["overshoots"])
    assert all(_close(g, r, rel, slack) for g, r in zip(got, ref)), (got, ref)
    f, st = m.spectra(cfg.ilinestart, cfg.nlines, stats=True)
    assert np.array_equal(f, plain)
    assert st["overshoots"] == sum(got), (st["overshoots"], got)
    m.set_checks(False)
    assert m.spectra(cfg.ilinestart, 1, stats=True)[1]["overshoots"] == 0
    m.free()
    ctx.close()


@pytest.mark.gpu
def test_gpu_cube_counts_match_oracle(gpu_lib, oracle_lib, tmp_path):
    cfg, d = _model(tmp_path, "tiny_band", command=2, pv_nx=8, pv_ny=6, nlines=1, ilinestart=1)
    o = oracle_lib.Oracle(d)
    o.posvel(1, **o.pv)
    ref = o.overshoots()
    assert ref > 0
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    m.set_precision(1)
    st = m.posvel(1, 1, stats=True)[-1]
    assert _close(st["overshoots"], ref, 1e-4, 4), (st["overshoots"], ref)
    m.free()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,warn", [("tiny_band", True), ("tiny_line", False)])
def test_run_dir_log(gpu_lib, oracle_lib, model_dir, tmp_path, name, warn):
    d = str(tmp_path / name)
    shutil.copytree(model_dir(name), d)
    st = gpu_lib.run_dir(d)
    assert (st["overshoots"] > 0) == warn
    log = open(os.path.join(d, "radlite.log")).read().split("\n")
    start = log.index(" =========== RUN OF RADICAL ===========")
    assert log[start + 1] == " Action       : spectrum/image"
    assert " Quadrature                 (SRCQDR_PNT_2)" in log
    nr = len(np.loadtxt(os.path.join(d, "radius.inp"), skiprows=1))
    assert " frsize radius      = %12d" % nr in log
    w = log.index(" Warnings:")
    assert (log[w + 1] == " * During Short Characteristic integration     ") == warn
    assert (log[w + 1] == " <none>") == (not warn)
    assert log[-2] == " ========= END OF RUN RADLITE ========="
