"""Batched rendering (rl_batch_*): many uneven models, line ranges and cameras in one
launch sequence must give the spectra of the per-model entry point (rl_spectra).

Both paths run the same per-(line, channel) arithmetic and the same deterministic
reduction, so FP64 agrees to 1e-12 and FP32 to 1e-6 relative (the compiler may contract
the two inlined copies of the walk differently)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("tiny_line", {}, 1, 1),
    ("tiny_band", {}, 1, 6),
    ("tiny_band", {"incl_deg": 20.0, "vmax": 10.0, "dv": 0.25}, 2, 5),
    ("small_line", {}, 2, 3),
    ("tiny_line", {"incl_deg": 80.0, "nphi": 8, "vmax": 30.0, "dv": 0.5}, 3, 2),
]


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _models(ctx, model_dir):
    out = []
    for name, over, il0, nl in CASES:
        m = ctx.load_dir(model_dir(name, **over))
        out.append((m, il0, nl))
    return out


@pytest.mark.parametrize("prec,tol", [(0, 1e-6), (1, 1e-12)])
def test_batch_matches_per_model(gpu_lib, ctx, model_dir, prec, tol):
    models = _models(ctx, model_dir)
    refs = []
    for m, il0, nl in models:
        m.set_precision(prec)
        refs.append(m.spectra(il0, nl))
    b = gpu_lib.Batch(ctx, precision=prec)
    for m, il0, nl in models:
        b.add(m, il0, nl)
    first, st = b.run(stats=True)
    again = b.run()          # graph replay
    assert st["ray_channels"] == sum(m.info()["nrays"] * m.info()["nfr"] * nl for m, _, nl in models)
    for got, got2, ref in zip(first, again, refs):
        assert got.shape == ref.shape
        np.testing.assert_array_equal(got, got2)
        for k in range(ref.shape[0]):
            assert relerr(got[k], ref[k]) <= tol, (k, relerr(got[k], ref[k]))
    b.close()
    for m, _, _ in models:
        m.free()


def test_batch_waves_tiles_and_eager(gpu_lib, ctx, model_dir):
    models = _models(ctx, model_dir)
    b = gpu_lib.Batch(ctx)
    for m, il0, nl in models:
        b.add(m, il0, nl)
    ref = b.run()
    assert b.waves() == 1
    # a small memory budget splits the jobs into several waves over one arena
    b.set_memory(4 << 20)
    got = b.run()
    assert b.waves() > 1
    for g, r in zip(got, ref):
        np.testing.assert_allclose(g, r, rtol=1e-6)
    # every tile shape gives the same spectra; the tuner keeps a valid one
    for lines, slots in ((1, 2), (3, 4), (8, 8), (32, 4)):
        b.set_tiles(lines, slots)
        assert b.tiles() == (lines, slots)
        for g, r in zip(b.run(), ref):
            np.testing.assert_allclose(g, r, rtol=1e-6)
    tune = b.autotune(sample_stride=3)
    assert tune["lines_per_item"] in (2, 8, 16, 32) and tune["channel_slots"] == 4
    assert tune["sample_ms"] > 0
    b.use_graph(False)
    for g, r in zip(b.run(), ref):
        np.testing.assert_allclose(g, r, rtol=1e-6)
    b.close()
    for m, _, _ in models:
        m.free()


def test_batch_rejects_bad_jobs(gpu_lib, ctx, model_dir):
    m = ctx.load_dir(model_dir("tiny_line"))
    b = gpu_lib.Batch(ctx)
    with pytest.raises(gpu_lib.RLError, match="line range"):
        b.add(m, 0, 1)
    with pytest.raises(gpu_lib.RLError, match="no jobs"):
        b.run()
    with pytest.raises(gpu_lib.RLError, match="lines_per_item"):
        b.set_tiles(33, 4)
    b.close()
    m.free()


def test_manifest_writes_the_per_directory_outputs(gpu_lib, model_dir, tmp_path):
    import os
    import shutil
    import subprocess
    names = [("tiny_line", {}), ("tiny_band", {}), ("small_line", {})]
    one, many = [], []
    for i, (name, over) in enumerate(names):
        src = model_dir(name, **over)
        a, b = str(tmp_path / f"one{i}"), str(tmp_path / f"many{i}")
        shutil.copytree(src, a)
        shutil.copytree(src, b)
        gpu_lib.run_dir(a)
        one.append(a)
        many.append(b)
    man = tmp_path / "models.txt"
    man.write_text("# model directories\n" + "\n".join(many) + "\n")
    r = subprocess.run([gpu_lib.EXE_PATH, "--manifest", str(man)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for a, b in zip(one, many):
        assert os.path.exists(os.path.join(b, "radlite.success"))
        fa = gpu_lib.read_spectrum_file(os.path.join(a, "linespectrum_moldata.dat"))
        fb = gpu_lib.read_spectrum_file(os.path.join(b, "linespectrum_moldata.dat"))
        assert len(fa) == len(fb)
        for x, y in zip(fa, fb):
            np.testing.assert_array_equal(x["velo"], y["velo"])
            np.testing.assert_allclose(y["flux"], x["flux"], rtol=2e-6)
    man.write_text(str(tmp_path / "missing") + "\n")
    r = subprocess.run([gpu_lib.EXE_PATH, "--manifest", str(man)], capture_output=True, text=True)
    assert r.returncode == 13
