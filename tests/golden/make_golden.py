"""Writes the golden spectra of the small synthetic models from the FP64 oracle.

Run from the repository root: python tests/golden/make_golden.py
Each fixture records the generator configuration and, per line, the oracle's F_nu at 1 pc,
the output-file velocities and the step counts. The models are regenerated from the
configuration (seeded), so only these small JSON files are committed."""
import json
import os
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from radlite_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402

CASES = [("tiny_line", {}), ("tiny_band", {}), ("small_line", {}), ("tiny_line", {"incl_deg": 5.0}),
         ("tiny_line", {"outer_bc": 2, "incl_deg": 80.0}), ("tiny_band", {"outer_bc": 3})]


def case_name(name, over):
    return name + "".join(f"_{k}{v:g}" for k, v in sorted(over.items()))


def main():
    pyoracle.build()
    for name, over in CASES:
        cfg = synth.config_by_name(name, **over)
        with tempfile.TemporaryDirectory() as d:
            synth.write_model(cfg, d)
            o = pyoracle.Oracle(d)
            lines = []
            for il in range(o.ilinestart, o.ilinestart + o.nlines_spec):
                flux, velo, cnt = o.line_spectrum(il)
                lines.append({"iline": il, "flux": [float(f"{x:.15e}") for x in flux],
                              "velo": [float(f"{x:.15e}") for x in velo], "counts": cnt})
        out = {"config": cfg.to_dict(), "nrays": o.nrays, "nfr": o.nfr, "lines": lines}
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), case_name(name, over) + ".json")
        with open(path, "w") as fh:
            json.dump(out, fh, indent=0)
        print("wrote", path)


if __name__ == "__main__":
    main()
