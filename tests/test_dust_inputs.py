"""Dust opacity files with temperature ranges ("-1 nfreq" header, read_dustopac_file,
dust.F:320-480; the reference is built with DUST_OPAC_TEMPDEP). The line dust reads the
first table only (dust_kappawgt_abs(.,1,.,.), line.F:3582-3605), so a file whose first range
holds the plain table renders the plain model. Host only."""
import os

import numpy as np
import pytest

from radlite_gb300 import synth


def model(tmp_path, tag):
    cfg = synth.config_by_name("tiny_line")
    return cfg, synth.write_model(cfg, str(tmp_path / tag))


def rewrite_with_ranges(d, ranges, scale2=3.0):
    """dustopac_1.inp as a temperature-range file: the plain table for the first range,
    scale2 times it for the others."""
    p = os.path.join(d, "dustopac_1.inp")
    rows = open(p).read().split("\n")
    nf, nsize = (int(x) for x in rows[0].split())
    vals = [float(x) for r in rows[1:] for x in r.split()]
    assert len(vals) == 2 * nf * nsize
    out = [f"{-1:12d}{nf:12d}", f"{nsize:12d}{0:12d}{len(ranges):12d}"]
    for k, (a, b) in enumerate(ranges):
        out.append(f"{a:.6e} {b:.6e}")
        f = 1.0 if k == 0 else scale2
        out += ["%.10e" % (f * v) for v in vals]
    open(p, "w").write("\n".join(out) + "\n")


def test_first_range_is_the_line_dust(oracle_lib, gpu_lib, tmp_path):
    cfg, d0 = model(tmp_path, "plain")
    _, d1 = model(tmp_path, "ranges")
    rewrite_with_ranges(d1, [(0.0, 150.0), (150.0, 1500.0), (1500.0, 1e33)])
    f0, _, c0 = oracle_lib.Oracle(d0).line_spectrum(cfg.ilinestart)
    f1, _, c1 = oracle_lib.Oracle(d1).line_spectrum(cfg.ilinestart)
    assert np.array_equal(f0, f1) and c0 == c1
    m0, m1 = gpu_lib.load_dir_host(d0), gpu_lib.load_dir_host(d1)
    assert m0.checksum() == m1.checksum()
    m0.free()
    m1.free()


@pytest.mark.parametrize("ranges,what", [([(10.0, 150.0)], "gap"), ([(0.0, 150.0), (200.0, 1e33)], "gap"),
                                         ([(0.0, 150.0), (100.0, 1e33)], "overlap")])
def test_bad_temperature_ranges_rejected(oracle_lib, gpu_lib, tmp_path, ranges, what):
    _, d = model(tmp_path, "bad")
    rewrite_with_ranges(d, ranges)
    with pytest.raises(Exception, match=what):
        oracle_lib.Oracle(d)
    with pytest.raises(gpu_lib.RLError, match=what):
        gpu_lib.load_dir_host(d)
