"""Outer boundary type 3: every circular-image ray starts at the interstellar field of
interstellfield.inp interpolated at its channel frequency (read_interstellfield,
star.F:690-727; line_init_passband_outerbc, line.F:3855-3903; charintline,
telescope.F:4016-4023). The position-velocity path never fills that table, so its rays
start from zeros (calc_write_line_posvel, telescope.F:1828-1924).

CPU: the oracle is linear in the field strength, ignores a zero field, zeroes the channels
whose bracket index equals the channel count (the reference's test against freq_nr), and
the readers reject a missing or inconsistent file. GPU: the library's spectra, batched
spectra, position-velocity cube and differentiable forward against the oracle and the
plain path."""
import os

import numpy as np
import pytest

from radlite_gb300 import synth


def write(tmp_path, tag, name="tiny_line", **over):
    cfg = synth.config_by_name(name, **over)
    return cfg, synth.write_model(cfg, str(tmp_path / tag))


def relerr(got, ref):
    sel = ref > 1e-3 * ref.max()
    return float(np.max(np.abs(got[sel] - ref[sel]) / np.abs(ref[sel])))


def test_oracle_field_strength_is_linear(oracle_lib, tmp_path):
    out = []
    for w in (1e-4, 1e-3, 4e-3):
        cfg, d = write(tmp_path, f"w{w}", outer_bc=3, isrf_w=w)
        f, _, cnt = oracle_lib.Oracle(d).line_spectrum(cfg.ilinestart)
        out.append((f, cnt))
    (f1, c1), (f2, c2), (f3, c3) = out
    assert c1 == c2 == c3
    pred = f1 + (4e-3 - 1e-4) / (1e-3 - 1e-4) * (f2 - f1)
    np.testing.assert_allclose(f3, pred, rtol=1e-10)
    assert np.all(f2 > f1)


def test_oracle_zero_field_is_black(oracle_lib, tmp_path):
    cfg, d0 = write(tmp_path, "bc0")
    _, d3 = write(tmp_path, "bc3", outer_bc=3, isrf_w=0.0)
    f0, _, c0 = oracle_lib.Oracle(d0).line_spectrum(cfg.ilinestart)
    f3, _, c3 = oracle_lib.Oracle(d3).line_spectrum(cfg.ilinestart)
    assert np.array_equal(f0, f3) and c0 == c3


def bracket_of_line(cfg):
    """1-based bracket index of the line centre in the dust frequency grid."""
    E, g, lines = synth.molecule_levels(cfg)
    nu = synth.line_freqs(cfg, E, lines)[cfg.ilinestart - 1]
    fr = synth.dust_frequency_grid(cfg, E, lines)
    return int(np.searchsorted(fr, nu))


def test_oracle_channel_count_quirk(oracle_lib, tmp_path):
    """Channel count equal to the line's bracket index: the reference zeroes every channel
    of the field (all channels share the bracket), so the spectrum is the black one."""
    base = synth.config_by_name("tiny_line")
    i = bracket_of_line(base)
    assert 3 <= i <= 20
    dv = 1.0
    vmax = (i - 1) * dv / 2.0 + 0.01            # INT(2 vmax / dv + 1) = i channels
    cfg, d0 = write(tmp_path, "bc0", vmax=vmax, dv=dv)
    _, d3 = write(tmp_path, "bc3", vmax=vmax, dv=dv, outer_bc=3)
    o0, o3 = oracle_lib.Oracle(d0), oracle_lib.Oracle(d3)
    assert o3.nfr == i
    f0, _, _ = o0.line_spectrum(cfg.ilinestart)
    f3, _, _ = o3.line_spectrum(cfg.ilinestart)
    assert np.array_equal(f0, f3)
    # one channel more: the field is back
    _, d4 = write(tmp_path, "bc3b", vmax=vmax + dv / 2.0, dv=dv, outer_bc=3)
    _, d5 = write(tmp_path, "bc0b", vmax=vmax + dv / 2.0, dv=dv)
    f4, _, _ = oracle_lib.Oracle(d4).line_spectrum(cfg.ilinestart)
    f5, _, _ = oracle_lib.Oracle(d5).line_spectrum(cfg.ilinestart)
    assert np.all(f4 > f5)


@pytest.mark.parametrize("damage", ["missing", "count"])
def test_readers_reject_bad_field_file(oracle_lib, gpu_lib, tmp_path, damage):
    _, d = write(tmp_path, "m", outer_bc=3)
    p = os.path.join(d, "interstellfield.inp")
    if damage == "missing":
        os.remove(p)
    else:
        rows = open(p).read().split("\n")
        rows[0] = "%12d" % (int(rows[0]) + 1)
        open(p, "w").write("\n".join(rows))
    with pytest.raises(Exception, match="interstellfield"):
        oracle_lib.Oracle(d)
    with pytest.raises(gpu_lib.RLError, match="interstellfield"):
        gpu_lib.load_dir_host(d)


def test_oracle_rejects_channels_above_the_table(oracle_lib, tmp_path):
    """Line 4 of the rotor lies above the dust frequencies (they cover lines 1-3): the
    reference would interpolate past the end of its table, the oracle stops."""
    cfg, d = write(tmp_path, "m", outer_bc=3)
    o = oracle_lib.Oracle(d)
    o.line_spectrum(cfg.ilinestart)
    with pytest.raises(Exception, match="above the last frequency"):
        o.line_spectrum(cfg.ilinestart + 1)


def test_oracle_posvel_needs_no_field_table(oracle_lib, tmp_path):
    """The position-velocity path never builds the field table, so a line above the
    frequency table renders there (and starts from zeros) where a spectrum stops."""
    cfg, d3 = write(tmp_path, "bc3", outer_bc=3)
    _, d0 = write(tmp_path, "bc0")
    size = 2.0 * float(synth.make_grid(cfg)[0][-1])
    i3, t3 = oracle_lib.Oracle(d3).posvel(cfg.ilinestart + 1, 6, 6, size, size, addstar=1)
    i0, t0 = oracle_lib.Oracle(d0).posvel(cfg.ilinestart + 1, 6, 6, size, size, addstar=1)
    assert np.array_equal(i3, i0) and np.array_equal(t3, t0)


def test_host_reader_takes_field(gpu_lib, tmp_path):
    _, d3 = write(tmp_path, "bc3", outer_bc=3)
    _, d0 = write(tmp_path, "bc0")
    m3, m0 = gpu_lib.load_dir_host(d3), gpu_lib.load_dir_host(d0)
    assert m3.info()["outer_bc"] == 3
    assert m3.checksum() != m0.checksum()
    m3.free()
    m0.free()


@pytest.mark.gpu
def test_gpu_field_spectra_match_oracle(gpu_lib, oracle_lib, tmp_path):
    """All lines of the band disk in one call (the per-channel table of each line sits
    behind the stellar one), FP32 and FP64, and the channel-count case."""
    cfg, d = write(tmp_path, "band", name="tiny_band", outer_bc=3)
    o = oracle_lib.Oracle(d)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    f32 = m.spectra(cfg.ilinestart, cfg.nlines)
    m.set_precision(1)
    f64, st = m.spectra(cfg.ilinestart, cfg.nlines, stats=True)
    integ = 0
    for k in range(cfg.nlines):
        ref, _, cnt = o.line_spectrum(cfg.ilinestart + k)
        assert relerr(f32[k], ref) <= 1e-4
        assert relerr(f64[k], ref) <= 1e-9
        integ += cnt["integrated"]
    assert st["integrated"] == integ
    m.free()
    base = synth.config_by_name("tiny_line")
    i = bracket_of_line(base)
    over = dict(vmax=(i - 1) / 2.0 + 0.01, dv=1.0)
    got = []
    for bc in (0, 3):
        c, dd = write(tmp_path, f"q{bc}", outer_bc=bc, **over)
        mm = ctx.load_dir(dd)
        got.append(mm.calc_line_spectrum(c.ilinestart)[0])
        mm.free()
    assert np.array_equal(got[0], got[1])
    ctx.close()


@pytest.mark.gpu
def test_gpu_rejects_channels_above_the_table(gpu_lib, tmp_path):
    cfg, d = write(tmp_path, "m", outer_bc=3)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    m.calc_line_spectrum(cfg.ilinestart)
    with pytest.raises(gpu_lib.RLError, match="above the last frequency"):
        m.calc_line_spectrum(cfg.ilinestart + 1)
    m.free()
    ctx.close()


@pytest.mark.gpu
def test_gpu_batch_with_field(gpu_lib, tmp_path):
    jobs = [write(tmp_path, "a", name="tiny_band", outer_bc=3), write(tmp_path, "b"),
            write(tmp_path, "c", outer_bc=3, isrf_w=4e-3)]
    ctx = gpu_lib.Context(0)
    models = [ctx.load_dir(d) for _, d in jobs]
    plain = [m.spectra(c.ilinestart, c.nlines) for (c, _), m in zip(jobs, models)]
    b = gpu_lib.Batch(ctx)
    for (c, _), m in zip(jobs, models):
        b.add(m, c.ilinestart, c.nlines)
    for got, ref in zip(b.run(), plain):
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)
    b.close()
    for m in models:
        m.free()
    ctx.close()


@pytest.mark.gpu
def test_gpu_posvel_ignores_field(gpu_lib, tmp_path):
    out = []
    for bc in (0, 3):
        cfg, d = write(tmp_path, f"pv{bc}", outer_bc=bc)
        ctx = gpu_lib.Context(0)
        m = ctx.load_dir(d)
        size = 2.2 * float(synth.make_grid(cfg)[0][-1])      # wider than the disk: empty pixels too
        m.set_posvel(16, 16, size, size, addstar=1)
        out.append(m.posvel(cfg.ilinestart, 1))
        m.free()
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    # a line above the frequency table: no field table, so the cube renders
    cfg, d = write(tmp_path, "pv_above", outer_bc=3)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    size = 2.0 * float(synth.make_grid(cfg)[0][-1])
    m.set_posvel(8, 8, size, size, addstar=1)
    m.posvel(cfg.ilinestart + 1, 1)
    m.free()
    ctx.close()


@pytest.mark.gpu
def test_gpu_diff_with_field(gpu_lib, tmp_path):
    """The differentiable forward starts from the field like the plain path, and its adjoint
    gives the directional derivative of the loss (central difference along a smooth
    direction of ln T)."""
    import torch
    cfg, d = write(tmp_path, "m", name="tiny_band", outer_bc=3)
    ctx = gpu_lib.Context(0)
    m = ctx.load_dir(d)
    m.set_precision(1)
    ref = m.spectra(cfg.ilinestart, cfg.nlines)
    lnT, lnX, b = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in synth.cell_params(cfg))
    dd = gpu_lib.Diff(m, cfg.ilinestart, cfg.nlines, precision=1)
    flux, st0 = dd.forward(lnT, lnX, b, stats=True)
    got = flux.cpu().numpy()
    # the plain path reads populations written from unrounded energies; the differentiable
    # one recomputes them from the molecule file's F12.4 energies
    for k in range(cfg.nlines):
        assert relerr(got[k], ref[k]) <= 1e-4
    target = dd.forward(lnT + 0.05, lnX, b * 1.05)
    scale = target.abs().max()

    def loss(f):
        return float((((f - target) / scale) ** 2).sum())

    flux = dd.forward(lnT, lnX, b)
    gT, _, _ = dd.backward(2.0 * (flux - target) / scale ** 2)
    r, t = np.meshgrid(np.linspace(0, 1, cfg.nr), np.linspace(0, 1, cfg.nt))
    v = torch.tensor(synth.cell_order(np.sin(3.0 * r) * np.cos(2.0 * t)), dtype=torch.float64, device="cuda")
    h = 1e-6
    lp_, stp = dd.forward(lnT + h * v, lnX, b, stats=True)
    lm_, stm = dd.forward(lnT - h * v, lnX, b, stats=True)
    assert (stp["steps"], stp["integrated"]) == (stm["steps"], stm["integrated"]) == (st0["steps"], st0["integrated"])
    fd = (loss(lp_) - loss(lm_)) / (2 * h)
    ad = float((gT * v).sum())
    assert abs(fd - ad) <= 1e-3 * abs(fd), (fd, ad)
    dd.close()
    m.free()
    ctx.close()
