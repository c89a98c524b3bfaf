"""Circular-image output of a SAVE_IMCIR build (telescope.F:1346-1373, 1594-1615): the
integration mask of the walk against the oracle's imcir_cmask, and RADlite_gpu's
lineposvelcirc files against the API image (the mask accumulates over the run's lines, as
the reference never clears imcir_cmask)."""
import os

import numpy as np
import pytest

from radlite_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def test_mask_matches_oracle(gpu_lib, oracle_lib, ctx, model_dir):
    d = model_dir("tiny_line")
    o = oracle_lib.Oracle(d)
    m = ctx.load_dir(d)
    m.set_precision(1)
    for iline in (1, 3):
        img, mask = m.line_image(iline, mask=True)
        ref, rmask, _ = o.line_image(iline)
        assert np.max(np.abs(img - ref)) <= 1e-9 * np.abs(ref).max()
        np.testing.assert_array_equal(mask[1:], rmask[1:])     # the central beam's mask is never written
        assert mask[1:].sum() < mask[1:].size                  # continuum copies exist
    m.free()


def test_run_dir_writes_imcir_files(gpu_lib, ctx, tmp_path):
    cfg = synth.config_by_name("tiny_line", nlines=2, ilinestart=1)
    d = synth.write_model(cfg, str(tmp_path / "m"))
    gpu_lib.run_dir(d, save_imcir=True)
    spec = gpu_lib.read_spectrum_file(os.path.join(d, "linespectrum_moldata.dat"))
    m = ctx.load_dir(d)
    info = m.info()
    nphi, nrr = info["nphi"], info["nrings"]
    sticky = None
    for iline in (1, 2):
        img, mask = m.line_image(iline, mask=True)
        sticky = mask if sticky is None else (sticky | mask)
        f = gpu_lib.read_imcir_file(os.path.join(d, f"lineposvelcirc_moldata_{iline}.dat"))
        assert (f["nfr"], f["nphi"], f["nrr"]) == (info["nfr"], nphi, nrr)
        rings = img[1:].reshape(nrr, nphi, -1).transpose(2, 1, 0)          # [nfr, nphi, nrr]
        np.testing.assert_allclose(f["image"], rings, rtol=6e-4, atol=1e-5 * np.abs(rings).max())
        np.testing.assert_allclose(f["central"], img[0], rtol=1e-15)
        np.testing.assert_array_equal(f["mask"], sticky[1:].reshape(nrr, nphi, -1).transpose(2, 1, 0))
        assert f["r"][-1] == 0.0 and np.all(np.diff(f["ri"]) > 0)
        assert abs(f["velo"][0] + f["velo"][-1]) < 1e-9 * abs(f["velo"][0])
        flux, _ = m.calc_line_spectrum(iline)
        np.testing.assert_allclose(spec[iline - 1]["flux"][::-1], flux, rtol=1e-5)
    m.free()
