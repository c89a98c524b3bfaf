"""Writes golden vectors of the spectrum post-processing (RadliteSpectrum.gen_spec) by
running the reference's own pyradlite code on seeded synthetic line profiles.

Run from the repository root, where the reference tree is present, naming the reference's
pyradlite package directory on the command line or in PYRADLITE_DIR:
    python tests/golden/make_genspec_golden.py <reference>/pyradlite/pyradlite

pyradlite imports astropy, matplotlib and its radmc helper at module level; none of them is
installed here and none is used by the two methods exercised (_read_core_radliteoutput,
_process_spectrum), so light stand-ins are registered before the import. The stand-in
speed of light is the exact SI value; the other constants feed only quantities that
the fixtures do not record. Each fixture stores its inputs (line profiles, parameters)
and the reference's outputs; only these small JSON files are committed."""
import json
import os
import sys
import tempfile
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def reference_path() -> str:
    """The reference's pyradlite package directory: argv[1], else $PYRADLITE_DIR."""
    p = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYRADLITE_DIR")
    if not p:
        sys.exit(f"usage: python {sys.argv[0]} <reference>/pyradlite/pyradlite  (or set PYRADLITE_DIR)")
    return p


def _stub_modules():
    class Q:
        def __init__(self, v):
            self.value = v
            self.cgs = self

    const = types.ModuleType("astropy.constants")
    for name, v in dict(c=2.99792458e10, u=1.66053906660e-24, au=1.495978707e13, G=6.6743e-8, m_p=1.67262192369e-24,
                        M_sun=1.988409870698051e33, R_sun=6.957e10, h=6.62607015e-27, k_B=1.380649e-16).items():
        setattr(const, name, Q(v))
    astropy = types.ModuleType("astropy")
    astropy.constants = const
    io = types.ModuleType("astropy.io")
    fits = types.ModuleType("astropy.io.fits")
    io.fits = fits
    astropy.io = io
    plt = types.ModuleType("matplotlib.pyplot")
    plt.cm = types.SimpleNamespace(bone_r=None)
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = plt
    radmc = types.ModuleType("radmc")
    for k, m in {"astropy": astropy, "astropy.constants": const, "astropy.io": io, "astropy.io.fits": fits,
                 "matplotlib": mpl, "matplotlib.pyplot": plt, "radmc": radmc}.items():
        sys.modules.setdefault(k, m)


def import_reference(path):
    _stub_modules()
    sys.path.insert(0, path)
    import radlite  # noqa: E402  (the reference module)
    return radlite


def synth_lines(seed, nlines, groups):
    """Line profiles as linespectrum files carry them: ascending velocities, E13.6 values.
    groups: list of (number of channels, vmax) per simulated output file."""
    rng = np.random.default_rng(seed)
    lines = []
    base = rng.uniform(2140.0, 2141.5, size=nlines)      # wavenumbers [cm^-1], close lines overlap
    for i in range(nlines):
        nch, vmax = groups[i % len(groups)]
        vel = np.linspace(-vmax, vmax, nch)
        sig = rng.uniform(2.0, 6.0)
        cont = rng.uniform(1e-20, 3e-20) * (1.0 + 0.002 * vel)
        flux = cont + rng.uniform(0.5, 5.0) * 1e-20 * np.exp(-(vel / sig) ** 2)
        r7 = lambda a: np.array([float("%.6e" % x) for x in a])
        lines.append({"vel": r7(vel), "flux": r7(flux), "freq": float(2.99792458e10 * base[i]),
                      "maxnumpoints": nch})
    return lines


CASES = [
    # name, seed, lines, channel groups (nch, vmax), obsres, vsampling, dist
    ("genspec_band", 3, 14, [(41, 20.0), (81, 20.0)], 3.0, 1.0, 140.0),
    ("genspec_even_kernel", 5, 6, [(49, 12.0)], 1.0, 1.0, 50.0),
    ("genspec_single", 7, 1, [(33, 8.0)], 0.4, 0.5, 1.0),
    ("genspec_overshoot", 5, 6, [(49, 12.0)], 1.0, 0.75, 50.0),
]


def process(radlite, lines, obsres, vsampling, dist):
    s = object.__new__(radlite.RadliteSpectrum)
    s._attrdict = {"units": {}, "verbose": False, "interpolation": "linear", "obsres": obsres,
                   "vsampling": vsampling, "dist": dist, "_radlitelineoutput": lines}
    s._process_spectrum()
    return {k: s.get_attr(k).tolist() for k in ("wavelength", "frequency", "spectrum", "emission", "continuum")}


def reader_case(radlite):
    """The reference's reader of one core's output: the linespectrum file the oracle writes
    (the reference's layout) and the moldata file of the synthetic model (pyradlite's
    layout)."""
    from oracle import pyoracle
    from radlite_gb300 import synth
    cfg = synth.config_by_name("tiny_band", nlines=3, nphi=8)
    with tempfile.TemporaryDirectory() as d:
        synth.write_model(cfg, d)
        pyoracle.build()
        pyoracle.run_dir(d)
        with open(os.path.join(d, "linespectrum_moldata.dat")) as fh:
            spec_text = fh.read()
        with open(os.path.join(d, "moldata.dat")) as fh:
            mol_text = fh.read()
        spec = os.path.join(d, "linespectrum_moldata_0.dat")
        molfile = os.path.join(d, "moldata_0.dat")
        with open(spec, "w") as fh:
            fh.write(spec_text)
        with open(molfile, "w") as fh:
            fh.write(mol_text)
        s = object.__new__(radlite.RadliteSpectrum)
        s._attrdict = {"units": {}, "verbose": False}
        out = s._read_core_radliteoutput({"spec": spec, "mol": molfile})
    conv = lambda v: v.tolist() if hasattr(v, "tolist") else v
    return {"spec_text": spec_text, "mol_text": mol_text,
            "line": [{k: conv(v) for k, v in ln.items()} for ln in out["line"]],
            "mol": [{k: conv(v) for k, v in m.items()} for m in out["mol"]]}


def main():
    radlite = import_reference(reference_path())
    here = os.path.dirname(os.path.abspath(__file__))
    for name, seed, n, groups, obsres, vsamp, dist in CASES:
        lines = synth_lines(seed, n, groups)
        try:
            out = process(radlite, [dict(x) for x in lines], obsres, vsamp, dist)
        except ValueError as e:   # the output grid overshoots the fine grid: the reference raises
            out = {"error": str(e)}
        fixture = {"params": {"obsres": obsres, "vsampling": vsamp, "dist": dist, "interpolation": "linear"},
                   "lines": [{k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in ln.items()} for ln in lines],
                   "out": out}
        with open(os.path.join(here, name + ".json"), "w") as fh:
            json.dump(fixture, fh)
        print("wrote", name, len(out.get("wavelength", [])), "output points", out.get("error", ""))
    with open(os.path.join(here, "genspec_reader.json"), "w") as fh:
        json.dump(reader_case(radlite), fh)
    print("wrote genspec_reader")


if __name__ == "__main__":
    main()
