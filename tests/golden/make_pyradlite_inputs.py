"""Writes tests/golden/pyradlite_band/: the input files that pyradlite itself writes for a
RADLite run (abundance, density, temperature, turbulence, velocity, radlite.inp,
linespectrum.inp, moldata.dat, levelpop_moldata.dat, levelpop.info), produced by running
pyradlite's own writer methods (radlite.py:1739-2230) and its LTE populations
(_prep_mol_forcore, radlite.py:1022-1121) on a small synthetic band disk.

Run from the repository root, where the reference tree is present:
    python tests/golden/make_pyradlite_inputs.py <reference>/pyradlite/pyradlite   (or set PYRADLITE_DIR)

The files pyradlite does not write (grid, dust, frequencies, star, line.inp) come from the
RADMC side of a real run; the tests take them from radlite_gb300.synth for the same model
(config.json). pyradlite's line list and partition-sum tables (HITRAN) are not available:
the line list is the synthetic band's (energies as the molecule file stores them) and the
partition sum is the sum over all of its levels, as for the LTE fixture."""
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from make_genspec_golden import import_reference, reference_path  # noqa: E402
from radlite_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "pyradlite_band")
# passband and sampling with two decimals: pyradlite writes them with {:<8.2f}
OVERRIDES = dict(nr=20, nt=10, nphi=16, vmax=12.0, dv=0.5, nrrextra=-6)
WRITTEN = ("abundance.inp", "density.inp", "temperature.inp", "turbulence.inp", "velocity.inp", "radlite.inp",
           "linespectrum.inp", "moldata.dat", "levelpop_moldata.dat", "levelpop.info")


class _Model:
    """The attributes pyradlite's writers and _prep_mol_forcore read, one core, all lines."""

    def __init__(self, attrs, hitran):
        self.attrs, self.hitran = attrs, hitran

    def get_attr(self, attrname):
        return self.attrs[attrname]

    def _get_core_attr(self, attrname, dictname=None, pind=0):
        return self.hitran[attrname]


def config():
    cfg = synth.config_by_name("tiny_band", **OVERRIDES)
    cfg.name = "pyradlite_band"
    return cfg


def main():
    radlite = import_reference(reference_path())
    cfg = config()
    f = synth.make_fields(cfg)
    E, g, lines = synth.molecule_levels(cfg)
    E = np.round(E, 4)
    nj = cfg.band_jmax_level + 1
    up = np.array([u - 1 for u, _, _ in lines])
    lo = np.array([l - 1 for _, l, _ in lines])
    vlab = np.array([f"v={i // nj}" for i in range(len(E))])
    jlab = np.array([f"J={i % nj}" for i in range(len(E))])
    hitran = {"Eup": E[up], "Elow": E[lo], "gup": g[up], "glow": g[lo], "wavenum": E[up] - E[lo],
              "A": np.array([a for _, _, a in lines]), "vup": vlab[up], "vlow": vlab[lo], "qup": jlab[up],
              "qlow": jlab[lo]}
    hck = radlite.h0 * radlite.c0 / radlite.kB0
    temp = f["temp"]
    psum = np.sum(g[:, None, None] * np.exp(-np.multiply.outer(E * hck, 1.0 / temp)), axis=0)
    with tempfile.TemporaryDirectory() as tmp:
        attrs = {"radius": f["r"], "theta": np.zeros(2 * cfg.nt), "gastemperature": temp, "gasdensity": f["rho"],
                 "abundance": f["abund"], "collpartner": 0.0, "turbulence": f["width"] * 1e5,
                 "velocity_radial": f["vel"][0], "velocity_theta": f["vel"][1], "velocity_phi": f["vel"][2],
                 "verbose": False, "_psum_interped": psum, "inp_path": tmp, "noisrf": cfg.outer_bc == 0,
                 "cir_np": cfg.nphi, "b_per_r": cfg.dbdr, "b_extra": cfg.nrrextra, "passband": cfg.vmax,
                 "vsampling": cfg.dv, "image": 0, "incl": cfg.incl_deg, "vlsr": 0.0, "molname": "band",
                 "molweight": cfg.mol_mass_amu}
        m = _Model(attrs, hitran)
        attrs["_levelpopdicts"] = [radlite.RadliteModel._prep_mol_forcore(m, 0)]
        M = radlite.RadliteModel
        for w in (M._write_abundanceinp, M._write_densityinp, M._write_gastemperatureinp, M._write_turbulenceinp,
                  M._write_velocityinp, M._write_radliteinp):
            w(m)
        M._write_core_linespectruminp(m, 0, tmp)
        M._write_core_moldatadat(m, tmp, 0)
        getattr(M._write_core_levelpopinp, "__wrapped__", M._write_core_levelpopinp)(m, tmp, 0)
        if os.path.isdir(OUT):
            shutil.rmtree(OUT)
        os.makedirs(OUT)
        for name in WRITTEN:
            shutil.copy(os.path.join(tmp, name), os.path.join(OUT, name))
    with open(os.path.join(OUT, "config.json"), "w") as fh:
        json.dump({"base": "tiny_band", "overrides": OVERRIDES, "written_by_pyradlite": list(WRITTEN)}, fh, indent=1)
    print("wrote", OUT, sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
