"""The bracketing search of the trajectory builder (hunt's index rules, nrecip.F:157-197)
in the product's geometry (rl_geometry.cuh, compiled for the host by tests/geom_host.cpp)
and in the oracle, against this file's own statement of the rules:

  past(j): x >= xx(j) (ascending table) / x < xx(j) (descending); before(j) the opposite
  comparison; beyond(j): x > xx(j) / x <= xx(j).
  Bracket [L, H] from the guess g by probes at distances 2^i - 1: upwards while past
  (L = last node passed, g at least; H = first probe not passed, n + 1 past the end),
  downwards while before (H = last such probe, g at least; L = first probe that is not,
  0 past the start); a guess outside 1..n gives [0, n + 1].
  Result: L + the number of nodes strictly inside the bracket that x lies beyond.

Exact hits on node values, guesses on every node and outside, ascending and descending
tables."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def hunt_rules(xx, x, g):
    n = len(xx)

    def X(j):
        return xx[j - 1]

    asc = X(n) > X(1)

    def past(j):
        return x >= X(j) if asc else x < X(j)

    def before(j):
        return x < X(j) if asc else x >= X(j)

    def beyond(j):
        return x > X(j) if asc else x <= X(j)

    lo, hi = 0, n + 1
    if 1 <= g <= n:
        d = 1
        if past(g):
            lo = g
            while g + d <= n:
                if not past(g + d):
                    hi = g + d
                    break
                lo = g + d
                d = 2 * d + 1
        else:
            hi = g
            while g - d >= 1:
                if not before(g - d):
                    lo = g - d
                    break
                hi = g - d
                d = 2 * d + 1
    return lo + sum(1 for j in range(lo + 1, hi) if beyond(j))


@pytest.fixture(scope="module")
def geom(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("geom") / "geom_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-x", "c++", os.path.join(HERE, "geom_host.cpp"),
                    "-o", so], check=True)
    L = C.CDLL(so)
    L.geom_hunt.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double, C.c_int]
    return L


def test_hunt_rules(geom, oracle_lib):
    lib = oracle_lib.lib()
    lib.rlo_hunt.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double, C.c_int]
    rng = np.random.default_rng(4)
    checked = 0
    for n in list(range(1, 13)) + [31, 64]:
        for order in (1, -1):
            xx = np.cumsum(rng.uniform(0.5, 2.0, n))
            if order < 0:
                xx = xx[::-1].copy()
            xs = list(xx) + list(0.5 * (xx[1:] + xx[:-1])) + [xx.min() - 1.0, xx.max() + 1.0]
            p = xx.ctypes.data_as(C.POINTER(C.c_double))
            for x in xs:
                for g in range(-1, n + 3):
                    want = hunt_rules(list(xx), float(x), g)
                    assert geom.geom_hunt(p, n, float(x), g) == want, (n, order, x, g)
                    assert lib.rlo_hunt(p, n, float(x), g) == want, (n, order, x, g)
                    checked += 1
    assert checked > 10000


def test_exact_hit_tie_rule():
    """Ascending table: an exact hit on node k returns k when the bracket stops on k, else k - 1."""
    xx = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0]
    assert hunt_rules(xx, 4.0, 4) == 4        # the guess itself
    assert hunt_rules(xx, 5.0, 4) == 5        # first upward probe (distance 1)
    assert hunt_rules(xx, 6.0, 4) == 5        # inside the bracket [5, 7]: the node below
    assert hunt_rules(xx, 7.0, 4) == 7        # probe at distance 3
    assert hunt_rules(xx, 4.0, 0) == 3        # no guess: bisection over [0, 9]
    assert hunt_rules(xx, 1.0, 0) == 0
