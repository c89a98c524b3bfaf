"""Seeded synthetic protoplanetary-disk models written in RADLite's input-file formats.

The reference ships no benchmark inputs, so every workload here is generated: a 2-D
axisymmetric (r, theta) disk with power-law surface density, Gaussian vertical structure,
radial temperature law, Keplerian rotation, grey dust, and either a pure rotational ladder
(a synthetic linear rotor) or a v=0-1 ro-vibrational band, with LTE level populations.

Formats follow the reference readers and the pyradlite writers:
  radius.inp           grid.F:716-727            theta.inp        grid.F:1103-1165
  density.inp          setup.F:1616-1672          velocity.inp     setup.F:776-785
  turbulence.inp       setup.F:825-843            abundance.inp    setup.F:903-911
  dustdens.inp         setup.F:525-670 (read_vector_field, isep=1)
  dusttemp.info / dusttemp_final.dat   setup.F:159-235, 295-420
  dustopac.inp / dustopac_1.inp        dust.F:92-447
  frequency.inp        grid.F:1445-1463           starinfo.inp     star.F:543-569
  starspectrum.inp     star.F:449-537             line.inp         line.F:142-367
  interstellfield.inp  star.F:690-727 (outer boundary 3)
  linespectrum.inp     telescope.F:86-257         moldata.dat      line.F:1826-1985
  levelpop.info / levelpop_moldata.dat line.F:811-950
  radlite.inp (format 104) main.F:488-686 + setup.F:1117-1137, template
                       pyradlite/pyradlite/radlite.py:2085-2150
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, asdict

import numpy as np

AU = 1.49597870e13
MSUN = 1.9891e33
RSUN = 6.9599e10
GRAV = 6.6726e-8
KB = 1.380658e-16
MP = 1.6726e-24
AMU = 1.6605402e-24
HPL = 6.6262e-27
CL = 2.99792458e10
PC = 3.08572e18
HC_K = 1.4387769          # hc/k [cm K]
DEBYE = 1.0e-18


@dataclass
class DiskConfig:
    """One synthetic model; defaults are the 100x60 single-line disk."""
    name: str = "disk_line"
    nr: int = 100
    nt: int = 60                      # stored theta points (upper half); mirrored about the midplane
    rin_au: float = 0.1
    rout_au: float = 100.0
    theta_open: float = 0.7           # grid spans pi/2-theta_open .. pi/2
    sigma0: float = 100.0             # g/cm^2 at 1 AU
    sigma_pow: float = -1.0
    h0: float = 0.05                  # H/R at 1 AU
    h_pow: float = 0.25
    t0: float = 1500.0                # K at t_r0_au
    t_pow: float = -0.5
    t_r0_au: float = 0.1
    mstar: float = 1.0                # Msun
    rstar_rsun: float = 2.0
    tstar: float = 4275.0
    abund: float = 1.0e-4
    gas_to_dust: float = 100.0
    kappa_abs: float = 1.0
    mol_mass_amu: float = 28.0
    turb_frac: float = 0.1            # turbulent width as a fraction of the sound speed
    molecule: str = "rotor"           # "rotor" (40-level J ladder) or "band" (v=0,1 ro-vibrational)
    nlev_rotor: int = 40
    rotor_b_ghz: float = 57.6
    rotor_dipole_debye: float = 0.11
    band_origin_cm: float = 2143.0
    band_a: float = 30.0
    band_jmax_level: int = 30
    band_nj: int = 10                 # P(1..nj) and R(1..nj)
    ilinestart: int = 3               # 1-based, as linespectrum.inp
    nlines: int = 1
    vmax: float = 20.0                # km/s, linespectrum.inp passband half width
    dv: float = 0.63                  # km/s
    incl_deg: float = 45.0
    nphi: int = 128
    dbdr: int = 3
    nrrextra: int = -93               # radlite.inp b_extra (negative: dynamic extra rays)
    perturb_sigma: float = 0.0        # lognormal sigma of per-cell T and rho factors
    seed: int = 0
    outer_bc: int = 0                 # 0 = black, 2 = CMB, 3 = interstellar field (interstellfield.inp)
    isrf_t: float = 6000.0            # outer boundary 3: diluted blackbody W B_nu(T) on frequency.inp
    isrf_w: float = 1.0e-3
    starpump: int = 1                 # 1 = read the stellar spectrum (central-ray star)
    nfreq_dust: int = 24
    # linespectrum.inp command 2 (position-velocity cube): pixels, full image size [AU],
    # rotation [rad], offsets [AU], unresolved-star flag
    command: int = 0
    pv_nx: int = 16
    pv_ny: int = 12
    pv_size_au: float = 0.0           # 0: the grid's outer diameter
    pv_phioff: float = 0.0
    pv_xoff_au: float = 0.0
    pv_yoff_au: float = 0.0
    pv_addstar: int = 1

    def to_dict(self):
        return asdict(self)


def config_by_name(name: str, **over) -> DiskConfig:
    """Named workloads: the reference-sized configurations and small test cases."""
    base = {
        # 100x60 disk, one rotor line, 64 channels, 400 rings x 128 azimuths
        "disk_line": dict(),
        # 400x200 perturbed disk, 20 band lines x 200 channels, 1000 rings x 256 azimuths
        "band_large": dict(name="band_large", nr=400, nt=200, perturb_sigma=0.1, seed=1,
                           molecule="band", ilinestart=1, nlines=20, vmax=24.875, dv=0.25,
                           nphi=256, dbdr=2, nrrextra=-192, incl_deg=20.0),
        # 200x100 disk, 10 rotor lines, 128 channels (INT(2 vmax/dv + 1) = INT(128.05)),
        # 600 rings x 128 azimuths
        "adjoint_disk": dict(name="adjoint_disk", nr=200, nt=100, ilinestart=1, nlines=10,
                             vmax=25.41, dv=0.4, nphi=128, dbdr=2, nrrextra=-192),
        # small cases that the FP64 oracle finishes in seconds
        "tiny_line": dict(name="tiny_line", nr=24, nt=12, nphi=16, dbdr=2, nrrextra=-6,
                          vmax=12.0, dv=0.75),
        "tiny_band": dict(name="tiny_band", nr=32, nt=16, perturb_sigma=0.1, seed=7,
                          molecule="band", band_nj=3, ilinestart=1, nlines=6, vmax=24.875,
                          dv=0.5, nphi=24, dbdr=2, nrrextra=-8, incl_deg=60.0),
        "small_line": dict(name="small_line", nr=60, nt=30, nphi=48, dbdr=2, nrrextra=-20,
                           ilinestart=2, nlines=3, vmax=15.0, dv=0.5),
    }
    if name not in base:
        raise KeyError(f"unknown workload {name!r}; known: {sorted(base)}")
    d = dict(base[name])
    d.update(over)
    return DiskConfig(**d)


def batch_configs(n: int = 256, seed: int = 2, nphi: int = 16) -> list:
    """The uneven multi-model workload: n seeded disks with nr ~ U[64,512], ntheta ~
    U[32,256], surface-density index ~ U[-1.5,-0.5], temperature index ~ U[-0.7,-0.3],
    stellar mass ~ U[0.3,2.5] Msun, inclination ~ U[5,85] deg, 1-50 lines of the
    ro-vibrational band (P and R branches, J = 1..25) and 32-256 channels. Channel counts
    come from (vmax, dv) pairs that satisfy the passband rule nfr = INT(2 vmax/dv + 1).
    Image radii follow the grid: dbdr 2 plus nr/4 extra inner rings, so there are
    2(nr-1) + 10 + nr/4 rings of nphi azimuths."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nr = int(rng.integers(64, 513))
        nt = int(rng.integers(32, 257))
        nch = int(rng.integers(32, 257))
        nl = int(rng.integers(1, 51))
        dv = 0.4
        out.append(DiskConfig(
            name=f"batch{i:03d}", nr=nr, nt=nt, sigma_pow=float(rng.uniform(-1.5, -0.5)),
            t_pow=float(rng.uniform(-0.7, -0.3)), mstar=float(rng.uniform(0.3, 2.5)),
            incl_deg=float(rng.uniform(5.0, 85.0)), molecule="band", band_nj=25, ilinestart=1,
            nlines=nl, dv=dv, vmax=((nch - 1) + 0.05) * dv / 2.0, nphi=nphi, dbdr=2,
            nrrextra=-max(8, nr // 4), seed=seed * 1000 + i))
    return out


# ----------------------------------------------------------------------------------------
# physical model on the stored grid
# ----------------------------------------------------------------------------------------

def make_grid(cfg: DiskConfig):
    r = np.exp(np.linspace(math.log(cfg.rin_au), math.log(cfg.rout_au), cfg.nr)) * AU
    j = np.arange(cfg.nt, dtype=np.float64)
    # IDL convention: last node half a step below pi/2 (PRO/problem_grid.pro:61-63)
    th = (0.5 * math.pi - cfg.theta_open) + cfg.theta_open * j / (cfg.nt - 0.5)
    return r, th


def molecule_levels(cfg: DiskConfig):
    """Return (E_cm [nlev], g [nlev], lines [(up, low, A)] 1-based)."""
    if cfg.molecule == "rotor":
        bcm = cfg.rotor_b_ghz * 1e9 / CL
        J = np.arange(cfg.nlev_rotor, dtype=np.float64)
        E = bcm * J * (J + 1.0)
        g = 2.0 * J + 1.0
        mu = cfg.rotor_dipole_debye * DEBYE
        lines = []
        for Ju in range(1, cfg.nlev_rotor):
            nu = 2.0 * cfg.rotor_b_ghz * 1e9 * Ju
            A = 64.0 * math.pi ** 4 * nu ** 3 / (3.0 * HPL * CL ** 3) * mu * mu * Ju / (2.0 * Ju + 1.0)
            lines.append((Ju + 1, Ju, A))
        return E, g, lines
    if cfg.molecule == "band":
        bcm = cfg.rotor_b_ghz * 1e9 / CL
        nj = cfg.band_jmax_level + 1
        E, g = [], []
        for v in (0, 1):
            for Jl in range(nj):
                E.append(v * cfg.band_origin_cm + bcm * Jl * (Jl + 1.0))
                g.append(2.0 * Jl + 1.0)
        E, g = np.array(E), np.array(g)
        lv = lambda v, Jl: v * nj + Jl + 1
        lines = []
        for Jl in range(1, cfg.band_nj + 1):        # P(J): (1, J-1) -> (0, J)
            lines.append((lv(1, Jl - 1), lv(0, Jl), cfg.band_a * Jl / (2.0 * Jl + 1.0)))
        for Jl in range(1, cfg.band_nj + 1):        # R(J): (1, J+1) -> (0, J)
            lines.append((lv(1, Jl + 1), lv(0, Jl), cfg.band_a * (Jl + 1.0) / (2.0 * Jl + 1.0)))
        return E, g, lines
    raise ValueError(cfg.molecule)


def make_fields(cfg: DiskConfig):
    """All per-cell arrays on the stored half grid, indexed [it, ir] like the reference."""
    r, th = make_grid(cfg)
    R2, T2 = np.meshgrid(r, th)                    # [nt, nr]
    Rcyl = R2 * np.sin(T2)
    z = R2 * np.cos(T2)
    sigma = cfg.sigma0 * (Rcyl / AU) ** cfg.sigma_pow
    H = cfg.h0 * (Rcyl / AU) ** cfg.h_pow * Rcyl
    rho = sigma / (math.sqrt(2.0 * math.pi) * H) * np.exp(-0.5 * (z / H) ** 2)
    temp = cfg.t0 * (R2 / (cfg.t_r0_au * AU)) ** cfg.t_pow
    if cfg.perturb_sigma > 0:
        rng = np.random.default_rng(cfg.seed)
        temp = temp * rng.lognormal(0.0, cfg.perturb_sigma, size=temp.shape)
        rho = rho * rng.lognormal(0.0, cfg.perturb_sigma, size=rho.shape)
    rho = np.maximum(rho, 1e-99)
    cs = np.sqrt(1.4 * KB * temp / (2.3 * MP))
    mmol = cfg.mol_mass_amu * AMU
    width = np.sqrt((cfg.turb_frac * cs) ** 2 + 2.0 * KB * temp / mmol) / 1e5      # km/s
    vphi = np.sqrt(GRAV * cfg.mstar * MSUN / R2)
    vel = np.stack([np.zeros_like(vphi), np.zeros_like(vphi), vphi], axis=0)    # [3, nt, nr]
    abund = np.full_like(rho, cfg.abund)
    E, g, lines = molecule_levels(cfg)
    ex = -np.multiply.outer(E * HC_K, 1.0 / temp)                            # [nlev, nt, nr]
    pop = g[:, None, None] * np.exp(ex - ex.max(axis=0, keepdims=True))
    pop = pop / pop.sum(axis=0, keepdims=True)
    return dict(r=r, theta=th, rho=rho, temp=temp, width=width, vel=vel, abund=abund,
                dust_rho=rho / cfg.gas_to_dust, dust_temp=temp.copy(), pop=pop,
                E=E, g=g, lines=lines)


def line_freqs(cfg: DiskConfig, E, lines):
    ev = 1.986468498e-16 * np.asarray(E)
    return np.array([1.509160e26 * (ev[u - 1] - ev[l - 1]) for (u, l, _) in lines])


def dust_frequency_grid(cfg: DiskConfig, E, lines):
    """Log-spaced dust frequencies covering every line from line 1 to the last requested
    one: a directory run renders lines 1.. whatever linespectrum.inp asks (main.F:204)."""
    nu = line_freqs(cfg, E, lines)
    sel = nu[0: cfg.ilinestart - 1 + cfg.nlines]
    lo, hi = 0.8 * sel.min(), 1.25 * sel.max()
    return np.exp(np.linspace(math.log(lo), math.log(hi), cfg.nfreq_dust))


def planck(nu, t):
    return 1.47455e-47 * nu ** 3 / np.expm1(4.7989e-11 * nu / t)


# ----------------------------------------------------------------------------------------
# writers (one function per reference file)
# ----------------------------------------------------------------------------------------

def _fmt_rows(arr, fmt="%.10e"):
    return "\n".join(fmt % v for v in np.asarray(arr).ravel()) + "\n"


def write_model(cfg: DiskConfig, outdir: str, fields: dict | None = None) -> str:
    """Write the model in the reference's file formats; `fields` replaces entries of
    make_fields() (e.g. temp, dust_temp, abund, width, pop on the [it, ir] grid)."""
    os.makedirs(outdir, exist_ok=True)
    f = make_fields(cfg)
    if fields:
        f.update(fields)
    nr, nt = cfg.nr, cfg.nt
    P = lambda name: os.path.join(outdir, name)

    with open(P("radius.inp"), "w") as fh:
        fh.write(f"{nr:12d}\n \n" + _fmt_rows(f["r"], "%.10e"))
    with open(P("theta.inp"), "w") as fh:
        fh.write(f"{nt:12d}{1:8d}\n \n" + _fmt_rows(f["theta"], "%.12f"))

    # fields: ir outer, it inner (setup.F:1658-1661)
    cell = lambda a: np.asarray(a).T.ravel()          # [nt,nr] -> ir-major
    with open(P("density.inp"), "w") as fh:
        fh.write(f"{nr}\t{nt}\t1\n" + _fmt_rows(cell(f["rho"]), "%.10e"))
    with open(P("temperature.inp"), "w") as fh:
        fh.write(f"{nr}\t{nt}\t1\n" + _fmt_rows(cell(f["temp"]), "%.8f"))
    v = f["vel"]
    with open(P("velocity.inp"), "w") as fh:
        fh.write(f"{nr}\t{nt}\n")
        rows = np.stack([cell(v[0]), cell(v[1]), cell(v[2])], axis=1)
        fh.write("\n".join("%.10e\t%.10e\t%.10e" % tuple(x) for x in rows) + "\n")
    with open(P("turbulence.inp"), "w") as fh:
        fh.write(f"1\n{nr}\t{nt}\n" + _fmt_rows(cell(f["width"]), "%.10e"))
    with open(P("abundance.inp"), "w") as fh:
        fh.write(f"{nr}\t{nt}\n")
        fh.write("\n".join("%.8e\t%.8f" % (a, 0.0) for a in cell(f["abund"])) + "\n")
    with open(P("dustdens.inp"), "w") as fh:
        fh.write(f"{1:12d}{nr:12d}{nt:12d}{1:8d}\n \n" + _fmt_rows(cell(f["dust_rho"]), "%.10e"))
    with open(P("dusttemp.info"), "w") as fh:
        fh.write("          -2\n           1\n           1\n           1\n           1\n")
    with open(P("dusttemp_final.dat"), "w") as fh:
        fh.write(f"{1:12d}{nr:12d}{nt:12d}{1:12d}\n\n{1:12d}\n" + _fmt_rows(cell(f["dust_temp"]), "%.12f"))

    E, g, lines = f["E"], f["g"], f["lines"]
    fr = dust_frequency_grid(cfg, E, lines)
    nf = len(fr)
    with open(P("frequency.inp"), "w") as fh:
        fh.write(f"{nf:12d}\n \n" + _fmt_rows(fr, "%.10e"))
    if cfg.outer_bc == 3:
        with open(P("interstellfield.inp"), "w") as fh:
            fh.write(f"{nf:12d}\n" + _fmt_rows(cfg.isrf_w * planck(fr, cfg.isrf_t), "%.10e"))
    with open(P("dustopac.inp"), "w") as fh:
        fh.write("2               Format number of this file\n"
                 "1               Nr of dust species\n"
                 "============================================================================\n"
                 "-1              Way in which this dust species is read (-1=file)\n"
                 "0               0=Thermal grain\n"
                 "1               Extension of name of dustopac_***.inp file\n"
                 "----------------------------------------------------------------------------\n")
    with open(P("dustopac_1.inp"), "w") as fh:
        fh.write(f"{nf:12d}{1:8d}\n \n" + _fmt_rows(np.full(nf, cfg.kappa_abs), "%.10e")
                 + " \n" + _fmt_rows(np.zeros(nf), "%.10e"))
    rstar = cfg.rstar_rsun * RSUN
    with open(P("starinfo.inp"), "w") as fh:
        fh.write(f"1\n   {rstar:.7e}\n   {cfg.mstar * MSUN:.7e}\n   {cfg.tstar:.4f}\n")
    fstar = math.pi * planck(fr, cfg.tstar) * rstar ** 2 / PC ** 2
    with open(P("starspectrum.inp"), "w") as fh:
        fh.write(f"{nf:12d}\n" + "\n".join("   %.7e   %.7e" % (a, b) for a, b in zip(fr, fstar)) + "\n")

    # line.inp: one full block for line 1, "same as previous" for the rest
    nl_all = len(lines)
    with open(P("line.inp"), "w") as fh:
        fh.write("2               Format number (1=<Apr06,2=>Apr06)\n1\t\tHow many molecule species\n"
                 "2.3\t\tAverage molecular weight\n"
                 "============================================================================\n")
        fh.write("----------------------------------------------------------------------------\n"
                 "1\t\tYes, specify info for line\n0\t\tSymmetry\n40\t\tNumber of frequency points\n"
                 "80.0e0\t\tWidth of line range (km/s)\n1\t\tLine profile\n0\t\tAdditional information\n")
        for _ in range(nl_all - 1):
            fh.write("----------------------------------------------------------------------------\n"
                     "0\t\tNo, Same as previous\n")

    # moldata.dat in the column formats read by line.F:1865-1935, with the extra columns
    # pyradlite writes and its spectrum reader uses (radlite.py:1981-2007, 2795-2823):
    # vibrational and rotational labels per level; wavenumber, E_up and labels per line
    if cfg.molecule == "band":
        nj = cfg.band_jmax_level + 1
        labels = [(f"v={i // nj}", f"J={i % nj}") for i in range(len(E))]
    else:
        labels = [("v=0", f"J={i}") for i in range(len(E))]
    with open(P("moldata.dat"), "w") as fh:
        fh.write(f"!MOLECULE\n{cfg.molecule}\n!MOLECULAR WEIGHT\n{cfg.mol_mass_amu:4.1f}\n"
                 f"!NUMBER OF ENERGY LEVELS\n{len(E):6d}\n!LEVEL + ENERGIES(cm^-1) + WEIGHT + v + Q\n")
        for i, (e, gg) in enumerate(zip(E, g)):
            fh.write(f"{i + 1:5d}{e:12.4f}{gg:7.1f}{labels[i][0]:>15s}{labels[i][1]:>15s}\n")
        fh.write(f"!NUMBER OF RADIATIVE TRANSITIONS\n{nl_all:6d}\n"
                 "!TRANS + UP + LOW + EINSTEINA(s^-1) + FREQ(cm^-1) + E_u(cm^-1) + v_l + Q_p + Q_pp\n")
        for i, (u, l, A) in enumerate(lines):
            wn = E[u - 1] - E[l - 1]
            fh.write(f"{i + 1:5d}{u:5d}{l:5d}{A:12.3e}{wn:16.7f}{E[u - 1]:12.5f}{labels[u - 1][0]:>15s}"
                     f"{labels[l - 1][0]:>15s}{labels[u - 1][1]:>15s}{labels[l - 1][1]:>15s}\n")

    pop = f["pop"]
    with open(P("levelpop.info"), "w") as fh:
        fh.write("-3\nlevelpop_moldata.dat\n0")
    with open(P("levelpop_moldata.dat"), "w") as fh:
        fh.write(f"{nr}\t{nt}\t{len(E)}\t1\n")
        fh.write("\t".join("%.10e" % x for x in E * HPL * CL) + "\n")
        fh.write("\t".join("%.1f" % x for x in g) + "\n")
        cells = pop.transpose(2, 1, 0).reshape(nr * nt, len(E))    # ir outer, it inner
        np.savetxt(fh, cells, fmt="%.10e", delimiter="\t")

    with open(P("linespectrum.inp"), "w") as fh:
        fh.write("1       Format number\n1       Spectrum output style\n" + "-" * 63 + "\n"
                 "2       Format number\n" + "-" * 63 + "\n"
                 f"{cfg.vmax:<8.3f}Width of line passband [km/s]\n"
                 f"{cfg.dv:<8.4f}Velocity sampling [km/s]\n" + "-" * 65 + "\n"
                 "2       Format number\nmoldata.dat\tMolecular data file\n"
                 f"{cfg.command:<8d}Command (0=spectrum, 2=image[3-D P/V cube])\n"
                 "1.0     Distance in [pc]\n"
                 f"{cfg.incl_deg:<8.3f}Inclination [deg]\n"
                 "0.0     Radial velocity, rel. to local standard of rest [km/s]\n"
                 f"{cfg.nlines:<8d}Nr of lines to make spectrum/image\n"
                 f"{cfg.ilinestart:<8d}Starting line to make spectrum/image\n")
        if cfg.command == 2:
            size = (cfg.pv_size_au * AU) if cfg.pv_size_au > 0 else 2.0 * float(f["r"][-1])
            fh.write(f"{cfg.pv_nx:<8d}Nr of x pixels\n{cfg.pv_ny:<8d}Nr of y pixels\n1       image size in cm?\n"
                     f"{size:.10e} size x direction\n{size * cfg.pv_ny / cfg.pv_nx:.10e} size y direction\n"
                     f"{cfg.pv_phioff:.10e} Phi offset?\n{cfg.pv_xoff_au * AU:.10e} x offset?\n"
                     f"{cfg.pv_yoff_au * AU:.10e} y offset?\n{cfg.pv_addstar:<8d}add star?\n")

    with open(P("radlite.inp"), "w") as fh:
        sep = "=" * 40 + "\n"
        fh.write("104\t\tInput format version\n" + sep +
                 "-1\t\tMaximum number; OBSOLETE NITER PARAMETER\n"
                 "2\t\tIteration method\n0\t\tFlux conservation trick\n"
                 "1.000e-06\t\tConvergence tolerance\n0\t\tConvergence crit type\n"
                 "1\t\tInitial guess type\n" + sep +
                 "41\t\tNr of mu-angle points\n16\t\tNr of phi-angle points\n"
                 "2\t\tType of mu gridding\n0.1\t\tLargest allowed error\n"
                 "1.0\t\tDmu wrt dR\n3\t\tExtra mus around mu=0\n" + sep +
                 f"{cfg.outer_bc}\t\tType of outer boundary\n"
                 "2\t\tType of inner boundary\n0\t\tType of equator boundary\n" + sep +
                 "57.3\t\tDefault inclination angle\n"
                 f"{cfg.nphi}\t\tNr Phi-points circular CCD\n"
                 f"{cfg.dbdr}\t\tThe number of b_i per r_i\n"
                 f"{cfg.nrrextra}\t\tThe number of extra b_i inside the inner radius\n" + sep +
                 "1\t\tSave NLTE\n0\t\tSave intensity at inu\n-1\t\tSave source at inu\n"
                 "0\t\tSave moments\n-1\t\tSave dusttemp/etc\n0\t\tSave ALI operator\n"
                 "1\t\tSave phys vars of medium\n0\t\tSave flux conservation data\n" + sep +
                 "-551\t\tType of setup\n0\t\tDo dust?\n1\t\tDo lines?\n"
                 "1\t\tInclude dust in lines?\n"
                 f"{cfg.starpump}\t\tInclude star pumping?\n" + sep)
    return outdir


def model_arrays(cfg: DiskConfig) -> dict:
    """The same model as write_model(), as in-memory arrays (no text round trip)."""
    f = make_fields(cfg)
    E, g, lines = f["E"], f["g"], f["lines"]
    fr = dust_frequency_grid(cfg, E, lines)
    rstar = cfg.rstar_rsun * RSUN
    fstar = math.pi * planck(fr, cfg.tstar) * rstar ** 2 / PC ** 2
    f.update(freq=fr, kappa_abs=np.full(len(fr), cfg.kappa_abs), kappa_scat=np.zeros(len(fr)),
             rstar=rstar, star_flux_1pc=fstar, cfg=cfg)
    return f


def cell_order(a):
    """[nt, nr] field -> the library's cell order (ir-1)*nth + (it-1)."""
    return np.asarray(a).T.ravel()


def cells_to_grid(a, cfg: DiskConfig):
    """The library's cell order (ir-1)*nth + (it-1) -> an [nt, nr] field (cell_order's inverse)."""
    return np.asarray(a).reshape(cfg.nr, cfg.nt).T.copy()


def lte_fields(cfg: DiskConfig, lnT, lnX, width) -> dict:
    """make_fields() entries for per-cell parameters of the differentiable raytrace (library
    cell order): gas and dust temperature, abundance, width, and the LTE populations the
    differentiable path derives from the temperature (lte_arrays' energies). With
    write_model(cfg, dir, fields=...) the reference's input files of that model."""
    E, g, _ = molecule_levels(cfg)
    T = cells_to_grid(np.exp(lnT), cfg)
    return dict(temp=T, dust_temp=T.copy(), abund=cells_to_grid(np.exp(lnX), cfg), width=cells_to_grid(width, cfg),
                pop=lte_populations(np.round(E, 4), g, T))


def cell_params(cfg: DiskConfig):
    """Per-cell parameters of the differentiable raytrace: ln T, ln abundance, width [km/s]."""
    f = make_fields(cfg)
    return (np.log(cell_order(f["temp"])), np.log(cell_order(f["abund"])), cell_order(f["width"]))


def lte_populations(E_cm, g, temp):
    """LTE level populations n_i = g_i exp(-E_i hc/kT) / Q, Q the sum over the given levels,
    values below 1e-99 set to 0 (pyradlite _prep_mol_forcore, radlite.py:1106-1118, with its
    interpolated partition-sum table replaced by the level sum). E_cm [nlev] in cm^-1, g
    [nlev], temp any shape; returns [nlev, *temp.shape]."""
    temp = np.asarray(temp, dtype=np.float64)
    ex = -np.multiply.outer(np.asarray(E_cm, dtype=np.float64) * HC_K, 1.0 / temp)
    lg = np.log(np.asarray(g, dtype=np.float64)).reshape((-1,) + (1,) * temp.ndim)
    m = (lg + ex).max(axis=0, keepdims=True)
    w = np.exp(lg + ex - m)
    pop = w / w.sum(axis=0, keepdims=True)
    pop[pop < 1e-99] = 0.0
    return pop


def lte_arrays(cfg: DiskConfig) -> dict:
    """model_arrays() with the level populations recomputed in LTE from the energies as the
    molecule file stores them (F12.4 cm^-1), i.e. the populations the differentiable
    raytrace derives from the temperature."""
    f = model_arrays(cfg)
    f["pop"] = lte_populations(np.round(f["E"], 4), f["g"], f["temp"])
    return f


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("name")
    ap.add_argument("outdir")
    ap.add_argument("--incl", type=float, default=None)
    a = ap.parse_args()
    over = {} if a.incl is None else {"incl_deg": a.incl}
    write_model(config_by_name(a.name, **over), a.outdir)
