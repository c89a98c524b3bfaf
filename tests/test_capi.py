"""The C-ABI library loads and exports every entry point that include/rlgpu.h declares;
host-side parsing of the input files works without a device."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "rlgpu.h")).read()
    return sorted(set(re.findall(r"^\s*int\s+(rl_\w+)\s*\(", src, flags=re.M)))


def test_header_symbols_exported(gpu_lib):
    L = gpu_lib.lib()
    names = declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(L, n), f"{n} declared in rlgpu.h but not exported"
    assert sorted(gpu_lib.EXPORTS) == names


def test_host_only_load_matches_files(gpu_lib, model_dir, oracle_lib):
    d = model_dir("tiny_band")
    m = gpu_lib.load_dir_host(d)
    info = m.info()
    o = oracle_lib.Oracle(d)
    assert (info["nr"], info["nth"], info["nfr"], info["nrays"]) == (o.nr, o.nth, o.nfr, o.nrays)
    assert info["nlines_spec"] == o.nlines_spec and info["ilinestart"] == o.ilinestart
    assert abs(info["aksmax"] - o.aksmax) <= 1e-12 * o.aksmax
    with pytest.raises(gpu_lib.RLError, match="device context"):
        m.calc_line_spectrum(1)


@pytest.mark.parametrize("fname,mutate,msg", [
    ("radius.inp", lambda t: "\n".join(t.split("\n")[:10]), "end of file"),
    ("theta.inp", lambda t: t.replace("       1\n", "       0\n", 1), "mirroring"),
    ("density.inp", lambda t: "3\t3\t1\n" + t.split("\n", 1)[1], "inconsistent"),
    ("levelpop.info", lambda t: "-3\nwrongname.dat\n0", "levelpop.info"),
    ("levelpop.info", lambda t: "-1\n", "cannot open"),
    ("linespectrum.inp", lambda t: t.replace("0       Command", "1       Command"), "command 1"),
    ("linespectrum.inp", lambda t: t.replace("0       Command", "2       Command"), "end of file"),
    ("radlite.inp", lambda t: t.replace("-551", "-500"), "setup type"),
    ("moldata.dat", lambda t: t.replace("    4    3", "    3    4"), "invalid levels"),
    ("velocity.inp", lambda t: t.replace("e+", "x+", 1), "not a number"),
])
def test_malformed_inputs_rejected(gpu_lib, tmp_path, fname, mutate, msg):
    from radlite_gb300 import synth
    d = synth.write_model(synth.config_by_name("tiny_line"), str(tmp_path / "m"))
    p = os.path.join(d, fname)
    txt = open(p).read()
    new = mutate(txt)
    assert new != txt
    open(p, "w").write(new)
    with pytest.raises(gpu_lib.RLError, match=msg):
        gpu_lib.load_dir_host(d)


def test_batch_and_diff_entry_points_check_arguments(gpu_lib):
    """The batched and differentiable entry points reject null handles on the host,
    before any device work (no GPU needed)."""
    import ctypes as C
    L = gpu_lib.lib()
    out = C.c_void_p()
    assert L.rl_batch_create(None, 0, C.byref(out)) == -1
    assert L.rl_batch_run(None, None, None) == -1
    assert L.rl_batch_add(None, None, 1, 1) == -1
    assert L.rl_batch_set_tiles(None, 1, 2) == -1
    assert L.rl_diff_create(None, 1, 1, 0, C.byref(out)) == -1
    assert L.rl_diff_forward(None, None, None, None, None, None) == -1
    assert L.rl_diff_backward(None, None, None, None, None, None) == -1
    assert L.rl_diff_set_checkpoint(None, 1) == -1
    assert L.rl_diff_batch_create(None, C.byref(out)) == -1
    assert L.rl_diff_batch_forward(None, None) == -1
    assert L.rl_run_manifest(None, 0, None) == -1
    assert "null" in gpu_lib._err()
    assert L.rl_run_dir_ex(b".", 0, 8, None) == -1 and "unknown flags" in gpu_lib._err()
    assert L.rl_posvel(None, 1, 1, None, None, None) == -1
    assert L.rl_gen_spec(None, None, None, None, None, None, None, None, None) == -1


def test_checks_setter(gpu_lib, model_dir):
    """rl_set_checks takes RL_CHECK_OVERSHOOT or 0 on a host-only model and rejects unknown
    flags and a null model (no GPU needed)."""
    m = gpu_lib.load_dir_host(model_dir("tiny_line"))
    m.set_checks(True)
    m.set_checks(False)
    L = gpu_lib.lib()
    assert L.rl_set_checks(m.h, 2) == -1 and "unknown flags" in gpu_lib._err()
    assert L.rl_set_checks(None, 1) == -1 and "null" in gpu_lib._err()


def _header_struct(name):
    """Field (name, C type) pairs of `typedef struct name { ... } name;` in rlgpu.h."""
    src = open(os.path.join(ROOT, "include", "rlgpu.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.match(r"(unsigned long long|double|int|const double\*|const int\*|const char\*) (.*)", decl)
        assert m, decl
        out += [(f.strip(), m.group(1)) for f in m.group(2).split(",")]
    return out


@pytest.mark.parametrize("cname,pyname", [("rl_stats", "Stats"), ("rl_model_info", "ModelInfo"),
                                          ("rl_model_arrays", "ModelArrays"), ("rl_posvel_spec", "PosvelSpec"),
                                          ("rl_genspec_lines", "GenspecLines"),
                                          ("rl_genspec_params", "GenspecParams")])
def test_struct_mirrors_match_header(gpu_lib, cname, pyname):
    """Each ctypes mirror of a structure of rlgpu.h has its fields, in order, with the same
    types."""
    import ctypes as C
    ctype = {"unsigned long long": C.c_ulonglong, "double": C.c_double, "int": C.c_int,
             "const double*": C.POINTER(C.c_double), "const int*": C.POINTER(C.c_int), "const char*": C.c_char_p}
    want = [(n, ctype[t]) for n, t in _header_struct(cname)]
    assert list(getattr(gpu_lib, pyname)._fields_) == want
