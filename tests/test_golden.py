"""Committed golden spectra (tests/golden/*.json, written by make_golden.py from the FP64
oracle): the oracle must keep reproducing them, and the GPU path must match them."""
import glob
import json
import os

import numpy as np
import pytest

from radlite_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.json"))
               if not os.path.basename(p).startswith(("genspec_", "lte_")))


def load(path):
    with open(path) as fh:
        g = json.load(fh)
    return g, synth.DiskConfig(**g["config"])


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-5] for p in CASES])
def test_oracle_reproduces_golden(oracle_lib, tmp_path, path):
    g, cfg = load(path)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    o = oracle_lib.Oracle(d)
    assert (o.nrays, o.nfr) == (g["nrays"], g["nfr"])
    for ln in g["lines"]:
        flux, velo, cnt = o.line_spectrum(ln["iline"])
        np.testing.assert_allclose(flux, ln["flux"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(velo, ln["velo"], rtol=1e-12, atol=1e-12)
        assert cnt == ln["counts"]


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-5] for p in CASES])
def test_gpu_matches_golden(gpu_lib, tmp_path, path):
    g, cfg = load(path)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    for ln in g["lines"]:
        ref = np.array(ln["flux"])
        got, _ = m.calc_line_spectrum(ln["iline"])
        assert relerr(got, ref) <= 1e-4
    m.set_precision(1)
    for ln in g["lines"]:
        ref = np.array(ln["flux"])
        got, _, st = m.calc_line_spectrum(ln["iline"], stats=True)
        assert relerr(got, ref) <= 1e-9
        assert st["integrated"] == ln["counts"]["integrated"]
    m.free()
    ctx.close()
