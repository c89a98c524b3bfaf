"""CPU restatement (numpy) of pyradlite's spectrum post-processing, RadliteSpectrum.gen_spec
(pyradlite/radlite.py:2420-2470): reading the per-core outputs (_read_core_radliteoutput,
radlite.py:2750-2878; _read_radliteoutput, 2881-2998) and building the observed spectrum
(_process_spectrum, 3001-3187).

Test infrastructure only: the tests and the CPU baseline compare the library's GPU
implementation with it. Pinned against the reference's own code run on seeded inputs
(tests/golden/genspec_*.json, written by tests/golden/make_genspec_golden.py)."""
from __future__ import annotations

import math
import os

import numpy as np

C0 = 2.99792458e10           # cm/s (radlite.py:45, astropy's exact value)
CINMU0 = C0 * 1.0e4          # micron/s (radlite.py:52)
CINKM0 = C0 / 1.0e5          # km/s (radlite.py:53)


def read_core(spec_path: str, mol_path: str):
    """(lines, mol) of one core: per line the velocities, fluxes and central frequency, and
    its molecular description (radlite.py:2780-2877)."""
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
    v = [x[24:39] for x in levels]
    q = [x[39:54] for x in levels]
    trans = [x.split() for x in mol[7 + nlev + 3:7 + nlev + 3 + ntrans]]
    nlines = int(spec[4])
    incl = float(spec[6].split()[2])
    maxnum = int(spec[5])
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
                     "Eup": float(t[5]), "vup": v[up], "vlow": v[lo], "qup": q[up], "qlow": q[lo]})
        i = i + 7 + npts - 1
    return lines, mols


def read_runs(run_paths):
    """All cores of all runs, duplicates removed, ordered as np.unique orders their keys
    (radlite.py:2899-2986)."""
    lines, mols = [], []
    for path in run_paths:
        names = os.listdir(path)
        specs = sorted(os.path.join(path, n) for n in names if n.startswith("linespectrum_moldata_") and n.endswith(".dat"))
        molfs = sorted(os.path.join(path, n) for n in names if n.startswith("moldata_") and n.endswith(".dat"))
        if len(specs) != len(molfs):
            raise ValueError(f"{path}: unequal numbers of spectrum and molecular data files")
        for s, m in zip(specs, molfs):
            ln, mo = read_core(s, m)
            lines += ln
            mols += mo
    keys = [d["molname"] + d["vup"] + d["vlow"] + d["qup"] + d["qlow"] + str(d["gup"]) + str(d["glow"]) + str(d["Eup"])
            for d in mols]
    idx = np.unique(keys, return_index=True)[1]
    lines = [lines[i] for i in idx]
    mols = [mols[i] for i in idx]
    if len({d["incl"] for d in mols}) > 1:
        raise ValueError("the runs do not all have the same inclination")
    return lines, mols


def _lin(x, xp, fp):
    """Linear interpolation inside [xp[0], xp[-1]] with np.interp's conventions (the
    reference's interp1d delegates linear float64 interpolation to it)."""
    if np.any(x < xp[0]) or np.any(x > xp[-1]):
        raise ValueError("a value in x_new is outside the interpolation range")
    return np.interp(x, xp, fp)


def _pairwise_sum(a):
    """numpy's pairwise summation order for a 1-D float64 array (np.sum)."""
    n = len(a)
    if n < 8:
        s = 0.0
        for v in a:
            s += v
        return s
    if n <= 128:
        r = [a[k] for k in range(8)]
        i = 8
        while i < n - (n % 8):
            for k in range(8):
                r[k] += a[i + k]
            i += 8
        s = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
        for v in a[i:]:
            s += v
        return s
    m = n // 2
    m -= m % 8
    return _pairwise_sum(a[:m]) + _pairwise_sum(a[m:])


def grids(lines, obsres: float, vsampling: float):
    """Box width, fine velocity step and the fine and output wavelength grids
    (radlite.py:3030-3069)."""
    maxvspan = max(abs(d["vel"][0]) for d in lines)
    boxwidth = max(3 * maxvspan, 3 * obsres)
    imax = int(np.argmax([d["maxnumpoints"] for d in lines]))
    vres = lines[imax]["vel"][1] - lines[imax]["vel"][0]
    freqs = np.array([d["freq"] for d in lines])
    freqs = freqs[freqs != 0]
    mu_lo = np.min(CINMU0 / 1.0 / freqs)
    mumin = mu_lo - (boxwidth * 1.0e9 * mu_lo / CINMU0)
    mu_hi = np.max(CINMU0 / 1.0 / freqs)
    mumax = mu_hi + (boxwidth * 1.0e9 * mu_hi / CINMU0)
    g = 1 + (vres / 1.0 / CINKM0)
    n = int(np.floor(np.log(mumax / 1.0 / mumin) / np.log(g)) + 1)
    fine = np.array([mumin * (g ** i) for i in range(n)])
    gu = 1 + (vsampling / 1.0 / CINKM0)
    nu = int(np.floor(np.log(mumax / 1.0 / mumin) / np.log(gu)) + 1)
    out = np.array([mumin * (gu ** i) for i in range(nu)])
    return boxwidth, vres, mumin, mumax, fine, out


def kernel(obsres: float, vres: float):
    """The Gaussian smoothing kernel (radlite.py:3141-3144) and numpy's sum of it."""
    n = np.ceil(3.0 * obsres / vres)
    top = -1 * 2 * ((np.arange(0, n) - ((n - 1) / 2.0)) ** 2)
    bot = ((obsres / 1.0 / vres) ** 2) * np.log(2.0)
    k = np.exp(top / bot)
    return k, _pairwise_sum(k)


def convolve_reflect(x, k):
    """scipy.ndimage.convolve(x, k, mode='reflect') for a symmetric 1-D kernel: the
    flipped kernel centred at len(k)//2, one sample to the left for even lengths, with
    half-sample symmetric edges (d c b a | a b c d | d c b a), repeated with period 2n for
    kernels that reach further than one grid length."""
    n, m = len(x), len(k)
    c = m // 2 - (1 if m % 2 == 0 else 0)
    kf = k[::-1]
    out = np.zeros(n)
    for j in range(m):
        idx = np.mod(np.arange(n) + j - c, 2 * n)
        idx = np.where(idx >= n, 2 * n - idx - 1, idx)
        out += x[idx] * kf[j]
    return out


def process(lines, obsres: float, vsampling: float, dist: float):
    """spectrum, emission, continuum [Jy at dist pc], wavelength [micron] and frequency
    [Hz] of the combined lines (radlite.py:3001-3187)."""
    boxwidth, vres, mumin, mumax, fine, outmu = grids(lines, obsres, vsampling)
    em_lines, cont_cen = [], []
    for d in lines:   # continuum through the two edge channels (radlite.py:3079-3089)
        xs = np.array([d["vel"][0], d["vel"][-1]])
        ys = np.array([d["flux"][0], d["flux"][-1]])
        em_lines.append(d["flux"] - _lin(d["vel"], xs, ys))
        cont_cen.append(float(_lin(np.array([0.0]), xs, ys)[0]))
    full_em = np.zeros(len(fine))
    for d, em in zip(lines, em_lines):   # radlite.py:3095-3114
        muold = (np.concatenate([[-1 * boxwidth], d["vel"], [boxwidth]]) * 1.0e9 / d["freq"]) + (CINMU0 / 1.0 / d["freq"])
        emold = np.concatenate([[em[0]], em, [em[-1]]])
        sel = np.where((fine <= muold[-1]) & (fine >= muold[0]))[0]
        full_em[sel] = full_em[sel] + _lin(fine[sel], muold, emold)
    mus = np.array([CINMU0 / 1.0 / d["freq"] for d in lines])
    order = np.argsort(mus, kind="stable")
    mus = np.concatenate([[mumin], mus[order], [mumax]])
    cs = np.array(cont_cen)[order]
    cs = np.concatenate([[cs[0]], cs, [cs[-1]]])
    full_cont = _lin(fine, mus, cs)
    full_em = full_em * 1.0e23 / (dist ** 2)
    full_cont = full_cont * 1.0e23 / (dist ** 2)
    full_y = full_cont + full_em
    k, ksum = kernel(obsres, vres)
    res_em = convolve_reflect(full_em, k) / 1.0 / ksum
    res_y = convolve_reflect(full_y, k) / 1.0 / ksum
    return {"wavelength": outmu, "frequency": C0 / (outmu * 1.0e-4), "spectrum": _lin(outmu, fine, res_y),
            "emission": _lin(outmu, fine, res_em), "continuum": _lin(outmu, fine, full_cont)}
