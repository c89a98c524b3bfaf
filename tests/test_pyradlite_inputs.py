"""A model directory whose line-side input files were written by pyradlite's own writer
methods (tests/golden/pyradlite_band/, made by make_pyradlite_inputs.py: abundance,
density, temperature, turbulence, velocity, radlite.inp, linespectrum.inp, moldata.dat with
only the levels its lines touch and the lines sorted by lower energy, levelpop files with
energies in erg). The grid, dust, frequency and star files, which a real run takes from
RADMC, come from synth for the same model.

* host: the library's reader takes the directory, with pyradlite's counts and camera;
* oracle: its spectra equal those of the same model written by synth, line for line
  (matched by wavenumber), to the precision of pyradlite's number formats;
* GPU: the library's spectra of the directory equal the oracle's (the parity bar)."""
import json
import os
import shutil

import numpy as np
import pytest

from radlite_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "pyradlite_band")


def compose(path):
    with open(os.path.join(FIX, "config.json")) as fh:
        meta = json.load(fh)
    cfg = synth.config_by_name(meta["base"], **meta["overrides"])
    d = synth.write_model(cfg, str(path))
    for name in meta["written_by_pyradlite"]:
        shutil.copy(os.path.join(FIX, name), os.path.join(d, name))
    return cfg, d


def wavenumbers(d):
    """Wavenumber [cm^-1] of each line of a moldata.dat, in file order."""
    with open(os.path.join(d, "moldata.dat")) as fh:
        rows = fh.read().splitlines()
    k = next(i for i, r in enumerate(rows) if r.startswith("!NUMBER OF RADIATIVE"))
    n = int(rows[k + 1])
    return [float(r.split()[4]) for r in rows[k + 3:k + 3 + n]]


def line_map(d_py, d_sy):
    """1-based synth line of each pyradlite line, by wavenumber."""
    wp, ws = wavenumbers(d_py), np.array(wavenumbers(d_sy))
    out = []
    for w in wp:
        j = int(np.argmin(np.abs(ws - w)))
        assert abs(ws[j] - w) < 1e-4
        out.append(j + 1)
    return out


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


def test_reader_takes_pyradlite_files(gpu_lib, tmp_path):
    cfg, d = compose(tmp_path / "py")
    m = gpu_lib.load_dir_host(d)
    info = m.info()
    m.free()
    assert info["nlev"] == 8                      # the levels the six lines touch
    assert info["nlines_mol"] == 6 and info["nlines_spec"] == 6 and info["ilinestart"] == 1
    assert info["nfr"] == int(2 * 12.0 / 0.5 + 1)
    assert (info["nr"], info["nth"], info["nphi"], info["dbdr"], info["nrrayextra"]) == (20, 10, 16, 2, -6)
    assert info["incl_deg"] == pytest.approx(60.0) and info["vmax"] == pytest.approx(12.0)
    assert info["outer_bc"] == 0


def test_oracle_pyradlite_files_equal_synth_files(oracle_lib, tmp_path):
    cfg, d_py = compose(tmp_path / "py")
    d_sy = synth.write_model(cfg, str(tmp_path / "sy"))
    o_py, o_sy = oracle_lib.Oracle(d_py), oracle_lib.Oracle(d_sy)
    assert (o_py.nrays, o_py.nfr) == (o_sy.nrays, o_sy.nfr)
    for i, j in enumerate(line_map(d_py, d_sy), start=1):
        fp, vp, _ = o_py.line_spectrum(i)
        fs, vs, _ = o_sy.line_spectrum(j)
        np.testing.assert_allclose(vp, vs, rtol=1e-9, atol=1e-9)
        # pyradlite's formats (%.8f temperatures and velocities, %.8e densities) and
        # hc/k's last digits in its LTE populations
        assert relerr(fp, fs) <= 1e-5


@pytest.mark.gpu
def test_gpu_matches_oracle_on_pyradlite_files(gpu_lib, oracle_lib, tmp_path):
    cfg, d = compose(tmp_path / "py")
    o = oracle_lib.Oracle(d)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    for i in range(1, 7):
        ref, _, cnt = o.line_spectrum(i)
        got, _ = m.calc_line_spectrum(i)
        assert relerr(got, ref) <= 1e-4
    m.set_precision(1)
    for i in range(1, 7):
        ref, _, cnt = o.line_spectrum(i)
        got, _, st = m.calc_line_spectrum(i, stats=True)
        assert relerr(got, ref) <= 1e-9
        assert st["integrated"] == cnt["integrated"]
    m.free()
    ctx.close()
