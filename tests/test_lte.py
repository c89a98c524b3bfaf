"""LTE level populations against pyradlite's own _prep_mol_forcore (radlite.py:1022-1121) on
the band molecule (tests/golden/lte_levels.json, written by make_lte_golden.py). The
populations are what the differentiable raytrace's table kernel (k_lte_lines) computes
on the device; the GPU tests show that kernel equals the plain path fed these
populations (synth.lte_arrays). Host only."""
import json
import os

import numpy as np

from radlite_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture():
    with open(os.path.join(HERE, "golden", "lte_levels.json")) as fh:
        return json.load(fh)


def level_index(d):
    E, g = np.array(d["E_cm"]), np.array(d["g"])
    idx = []
    for e, gg in zip(d["Euniq"], d["guniq"]):
        hit = np.flatnonzero((np.abs(E - e) <= 1e-4 * (e + 0.1)) & (g == gg))
        assert hit.size == 1
        idx.append(int(hit[0]))
    return np.array(idx)


def test_unique_levels_are_the_lines_levels():
    d = fixture()
    idx = level_index(d)
    touched = sorted({u - 1 for u, _ in d["lines"]} | {l - 1 for _, l in d["lines"]})
    assert sorted(idx.tolist()) == touched


def test_partition_sum_is_the_level_sum():
    d = fixture()
    E, g, T = np.array(d["E_cm"]), np.array(d["g"]), np.array(d["temp"])
    q = np.sum(g[:, None, None] * np.exp(-np.multiply.outer(E * synth.HC_K, 1.0 / T)), axis=0)
    np.testing.assert_allclose(q, np.array(d["psum"]), rtol=1e-6)


def test_populations_match_reference():
    d = fixture()
    idx = level_index(d)
    ref = np.array(d["npop"])
    T = np.array(d["temp"])
    ours = synth.lte_populations(d["E_cm"], d["g"], T)[idx]
    # hc/k: 1.4387769 here, 1.43877688 from the SI constants: E/kT up to ~700 makes the
    # relative difference of a population up to ~1e-5
    big = ref > 1e-90
    rel = np.abs(ours[big] - ref[big]) / ref[big]
    assert rel.max() < 2e-5, rel.max()
    # the 1e-99 trim: the same cells are zero except within the constants' difference of it
    edge = (np.maximum(ours, ref) > 1e-99 * (1 - 1e-4)) & (np.minimum(ours, ref) < 1e-99 * (1 + 1e-4))
    assert np.array_equal(ours == 0, ref == 0) or np.all(((ours == 0) == (ref == 0)) | edge)
    assert (ref == 0).sum() > 0 and (ref > 0).sum() > 0
