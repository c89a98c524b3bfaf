"""The fit's error split over the Gauss-Newton eigenvectors (host arithmetic only)."""
import math

import numpy as np


def test_error_in_eigenbasis():
    from radlite_gb300 import fit
    rng = np.random.default_rng(3)
    q, _ = np.linalg.qr(rng.normal(size=(4, 4)))
    lam = np.array([1e-8, 1e-3, 0.5, 40.0])
    gn = {"eigenvalues": [lam.tolist()], "vectors": [q.tolist()]}
    e0 = np.array([[0.15, 0.08, -0.4, 0.4]])
    e1 = 0.7 * q[:, 0] + 1e-3 * q[:, 3]
    out = fit.error_in_eigenbasis(gn, e0, e1[None, :])
    assert math.isclose(out["weak_component_end"][0], 0.7, rel_tol=1e-12)
    assert math.isclose(out["weak_component_start"][0], float(q[:, 0] @ e0[0]), rel_tol=1e-12)
    seen0 = math.sqrt(float(np.sum(lam * (q.T @ e0[0]) ** 2)))
    seen1 = math.sqrt(1e-8 * 0.49 + 40.0 * 1e-6)
    assert math.isclose(out["seen_error_start"][0], seen0, rel_tol=1e-12)
    assert math.isclose(out["seen_error_end"][0], seen1, rel_tol=1e-9)
    assert math.isclose(out["median_seen_error_ratio_end_over_start"], seen1 / seen0, rel_tol=1e-9)
