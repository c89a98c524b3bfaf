"""Writes the golden LTE level populations (tests/golden/lte_levels.json) by running
pyradlite's own _prep_mol_forcore (radlite.py:1022-1121) on the ro-vibrational band molecule
of the synthetic models.

Run from the repository root, where the reference tree is present:
    python tests/golden/make_lte_golden.py <reference>/pyradlite/pyradlite   (or set PYRADLITE_DIR)

pyradlite takes the unique levels from a HITRAN line list (lower and upper energies,
degeneracies and quantum numbers per line) and divides g exp(-E hc/kT) by a partition sum
interpolated from a HITRAN table. Neither table exists here, so the line list is the band
molecule's (energies as the molecule file stores them, F12.4 cm^-1) and the partition sum
handed to the method is the sum over all of the molecule's levels, the partition sum the
library uses. The fixture stores those inputs and the method's unique levels and
populations; the stand-in physical constants are the exact SI values (make_genspec_golden)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from make_genspec_golden import import_reference, reference_path  # noqa: E402
from radlite_gb300 import synth  # noqa: E402

CONFIG = "band_large"


class _Model:
    """The attributes _prep_mol_forcore reads, for one core holding every line."""

    def __init__(self, hitran, theta, temp, psum):
        self.hitran, self.attrs = hitran, {"theta": theta, "gastemperature": temp, "verbose": False,
                                           "_psum_interped": psum}

    def _get_core_attr(self, attrname, dictname, pind):
        return self.hitran[attrname]

    def get_attr(self, attrname):
        return self.attrs[attrname]


def inputs():
    cfg = synth.config_by_name(CONFIG)
    E, g, lines = synth.molecule_levels(cfg)
    E = np.round(E, 4)
    nj = cfg.band_jmax_level + 1
    up = np.array([u - 1 for u, _, _ in lines])
    lo = np.array([l - 1 for _, l, _ in lines])
    hitran = {"Eup": E[up], "Elow": E[lo], "gup": g[up], "glow": g[lo], "wavenum": E[up] - E[lo],
              "vup": up // nj, "vlow": lo // nj, "qup": up % nj, "qlow": lo % nj}
    # temperatures from 4 K (upper band levels trimmed below 1e-99) to 3000 K, on a 4 x 6
    # stored half of a 8 x 6 grid
    t = np.geomspace(4.0, 3000.0, 24).reshape(4, 6)
    temp = np.concatenate([t, t[::-1]], axis=0)
    return E, g, lines, hitran, temp


def main():
    radlite = import_reference(reference_path())
    E, g, lines, hitran, temp = inputs()
    hck = radlite.h0 * radlite.c0 / radlite.kB0
    half = temp[: temp.shape[0] // 2]
    psum = np.sum(g[:, None, None] * np.exp(-np.multiply.outer(E * hck, 1.0 / half)), axis=0)
    theta = np.zeros(temp.shape[0])
    out = radlite.RadliteModel._prep_mol_forcore(_Model(hitran, theta, temp, psum), 0)
    fixture = {"config": CONFIG, "hc_over_k": hck, "E_cm": E.tolist(), "g": g.tolist(),
               "lines": [[int(u), int(l)] for u, l, _ in lines], "temp": half.tolist(), "psum": psum.tolist(),
               "Euniq": np.asarray(out["Euniq"]).tolist(), "guniq": np.asarray(out["guniq"]).tolist(),
               "npop": np.asarray(out["npop"]).tolist()}
    with open(os.path.join(HERE, "lte_levels.json"), "w") as fh:
        json.dump(fixture, fh)
    print("wrote lte_levels", len(fixture["Euniq"]), "levels x", half.size, "cells")


if __name__ == "__main__":
    main()
