"""Spectrum post-processing with the same interface as pyradlite's RadliteSpectrum
(pyradlite/radlite.py:2226-3187): read the per-core line spectra of one or more RADLite
runs, drop duplicate lines, and combine them into one observed spectrum at a distance,
smoothed to an observing resolution and sampled at a velocity step.

The reading and de-duplication (radlite.py:2750-2998) are host work on the output files;
the combination (_process_spectrum, radlite.py:3001-3187) runs on the GPU through
rl_gen_spec. Only linear interpolation is supported (the reference's interp1d kinds other
than 'linear' are rejected).
"""
from __future__ import annotations

import json
import os

import numpy as np

C0 = 2.99792458e10           # cm/s


def read_core(spec_path: str, mol_path: str):
    """Line profiles and molecular descriptions of one core's output pair,
    linespectrum_moldata_<i>.dat and moldata_<i>.dat (radlite.py:2780-2877)."""
    with open(spec_path) as fh:
        spec = fh.readlines()
    with open(mol_path) as fh:
        mol = fh.readlines()
    molname = mol[1].split("\n")[0]
    molweight = float(mol[3])
    nlev = int(mol[5])
    ntrans = int(mol[7 + nlev + 1])
    levels = mol[7:7 + nlev]
    g = [float(x[17:24]) for x in levels]
    vlab = [x[24:39] for x in levels]
    qlab = [x[39:54] for x in levels]
    trans = [x.split() for x in mol[7 + nlev + 3:7 + nlev + 3 + ntrans]]
    nlines = int(spec[4])
    maxnum = int(spec[5])
    incl = float(spec[6].split()[2])
    lines, mols = [], []
    i = 6
    for a in range(nlines):
        t = trans[a]
        wavenum = float(t[4])
        freq = C0 / (1.0 / wavenum)
        npts = int(spec[i + 5])
        rows = np.array([r.split() for r in spec[i + 7:i + 7 + npts]]).astype(float)
        lines.append({"vel": rows[:, 0], "flux": rows[:, 1], "freq": freq, "maxnumpoints": maxnum})
        up, lo = int(t[1]) - 1, int(t[2]) - 1
        mols.append({"molname": molname, "molweight": molweight, "incl": incl, "gup": g[up], "glow": g[lo],
                     "A": float(t[3]), "wavenum": wavenum, "wavelength": C0 / 1.0 / freq, "freq": freq,
                     "Eup": float(t[5]), "vup": vlab[up], "vlow": vlab[lo], "qup": qlab[up], "qlow": qlab[lo]})
        i = i + 7 + npts - 1
    return lines, mols


def read_runs(run_paths):
    """Every core of every run, duplicates removed (the kept lines are ordered as
    np.unique orders their identity keys, radlite.py:2961-2973); all runs must share one
    inclination."""
    lines, mols = [], []
    for path in run_paths:
        names = os.listdir(path)
        specs = sorted(os.path.join(path, n) for n in names
                       if n.startswith("linespectrum_moldata_") and n.endswith(".dat"))
        molfs = sorted(os.path.join(path, n) for n in names if n.startswith("moldata_") and n.endswith(".dat"))
        if len(specs) != len(molfs):
            raise ValueError(f"{path} does not hold as many spectrum as molecular data files")
        for sp, mo in zip(specs, molfs):
            ln, md = read_core(sp, mo)
            lines += ln
            mols += md
    keys = [d["molname"] + d["vup"] + d["vlow"] + d["qup"] + d["qlow"] + str(d["gup"]) + str(d["glow"]) + str(d["Eup"])
            for d in mols]
    keep = np.unique(keys, return_index=True)[1]
    lines = [lines[k] for k in keep]
    mols = [mols[k] for k in keep]
    if len({d["incl"] for d in mols}) > 1:
        raise ValueError("the RADLite runs do not all have the same source inclination")
    return lines, mols


class RadliteSpectrum:
    """pyradlite's RadliteSpectrum: parameters from a JSON file of {name: {"value": v}}
    (or a dict), gen_spec() to build the spectrum, get_attr() to read it."""

    def __init__(self, infile, ctx=None):
        if isinstance(infile, dict):
            params = dict(infile)
        else:
            with open(infile) as fh:
                params = {k: v["value"] for k, v in json.load(fh).items()}
        self._attrdict = dict(params)
        self._attrdict["units"] = {}
        self._ctx = ctx
        kind = self._attrdict.get("interpolation", "linear")
        if kind != "linear":
            raise ValueError(f"interpolation {kind!r}: only 'linear' is supported")

    def get_attr(self, name):
        return self._attrdict[name]

    def get_unit(self, name):
        return self._attrdict["units"][name]

    def gen_spec(self):
        from . import Context
        lines, mols = read_runs(self.get_attr("run_paths"))
        self._attrdict["_radlitelineoutput"] = lines
        self._attrdict["molinfo"] = mols
        ctx = self._ctx or Context(0)
        out = ctx.gen_spec(lines, self.get_attr("obsres"), self.get_attr("vsampling"), self.get_attr("dist"))
        units = {"spectrum": "Jy", "emission": "Jy", "continuum": "Jy", "wavelength": "micron", "frequency": "Hz"}
        for k, u in units.items():
            self._attrdict[k] = out[k]
            self._attrdict["units"][k] = u
        if self._ctx is None:
            ctx.close()
