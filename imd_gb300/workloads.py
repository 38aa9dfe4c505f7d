"""Synthetic inputs in IMD's own file formats.

The reference (itapmd/imd) ships no potentials, configurations or
benchmarks, so every workload is generated here, deterministically and
seeded:

* potential tables in IMD table format 2 (header ``#F 2 <ncols>``, then per
  column ``begin end step`` on r^2, then the values; read by
  src/imd_potential.c:394-462) -- a Lennard-Jones pair table and
  Sutton-Chen EAM2 tables (pair phi, density rho, embedding F);
* IMD parameter files (tokens parsed by src/imd_param.c:251 onwards) and
  configuration files (``#F A 1 1 1 3 3 0`` header, src/imd_io.c:3369);
* fcc crystals with Maxwell momenta, and batches of strained defect cells.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# units of IMD's eV / Angstrom / amu system: one time unit is 10.18051 fs
FS = 1.0 / 10.18051
KB_EV = 8.617343e-5


@dataclass
class Species:
    """One Sutton-Chen species: phi = eps (a/r)^9, rho = (a/r)^6,
    F = -c eps sqrt(rho)."""
    eps: float
    c: float
    a: float
    mass: float


CU = Species(eps=1.2382e-2, c=39.432, a=3.61, mass=63.546)
NI = Species(eps=1.5707e-2, c=39.432, a=3.52, mass=58.69)


def _taper(r: np.ndarray, rc: float, width: float) -> np.ndarray:
    """Cubic taper 1 - 3x^2 + 2x^3 on [rc - width, rc], 1 below, 0 above."""
    x = np.clip((r - (rc - width)) / width, 0.0, 1.0)
    return 1.0 - 3.0 * x * x + 2.0 * x * x * x


def _fmt(v: float) -> str:
    return "%.17e" % v


def write_table2(path: str, begin, end, step, columns) -> None:
    """Write an IMD format-2 table: one (begin, end, step) line per column,
    then each column's values, separated by blank lines."""
    ncols = len(columns)
    with open(path, "w") as f:
        f.write("#F 2 %d\n#E\n" % ncols)
        for c in range(ncols):
            f.write("%s %s %s\n" % (_fmt(begin[c]), _fmt(end[c]), _fmt(step[c])))
        for c in range(ncols):
            f.write("\n".join(_fmt(v) for v in columns[c]))
            f.write("\n\n")


def write_table1(path: str, r2, columns) -> None:
    """Write an IMD format-1 table: lines ``r2 v_0 ... v_{ncols-1}``."""
    with open(path, "w") as f:
        f.write("#F 1 %d\n#E\n" % len(columns))
        for k in range(len(r2)):
            f.write(" ".join(_fmt(v) for v in [r2[k]] + [c[k] for c in columns]) + "\n")


def lj_table(path: str, eps: float = 1.0, sigma: float = 1.0, rc: float = 2.5,
             rmin: float = 0.8, npts: int = 1000, fmt: int = 2) -> None:
    """Lennard-Jones 4 eps ((s/r)^12 - (s/r)^6) on r^2 from rmin^2 to rc^2.
    The reader shifts it to zero at the cutoff (src/imd_potential.c:439-450)."""
    r2 = np.linspace(rmin * rmin, rc * rc, npts)
    sr6 = (sigma * sigma / r2) ** 3
    v = 4.0 * eps * (sr6 * sr6 - sr6)
    if fmt == 2:
        step = (rc * rc - rmin * rmin) / (npts - 1)
        write_table2(path, [rmin * rmin], [rc * rc], [step], [v])
    else:
        write_table1(path, r2, [v])


def sutton_chen_tables(prefix: str, species: list[Species], rc: float = 7.2,
                       taper: float = 0.3, rmin: float = 1.5, npts: int = 2000,
                       rho_max: float = 400.0, nrho: int = 2000) -> tuple[str, str, str]:
    """EAM2 tables for a Sutton-Chen alloy.

    Pair column it*nt+jt: eps_ij (a_ij/r)^9 with eps_ij the geometric and a_ij
    the arithmetic mean.  Density column it*nt+jt is what an atom of type it
    receives from a neighbour of type jt (src/imd_forces_nbl.c:1176-1178):
    (a_jt/r)^6.  Embedding column t: -c_t eps_t sqrt(rho).  phi and rho carry
    a cubic taper over the last `taper` Angstrom before rc.
    Returns the (pair, rho, embed) file names."""
    nt = len(species)
    r2 = np.linspace(rmin * rmin, rc * rc, npts)
    r = np.sqrt(r2)
    s = _taper(r, rc, taper)
    step = (rc * rc - rmin * rmin) / (npts - 1)
    pair, dens = [], []
    for it in range(nt):
        for jt in range(nt):
            A, B = species[it], species[jt]
            eij = math.sqrt(A.eps * B.eps)
            aij = 0.5 * (A.a + B.a)
            pair.append(eij * (aij / r) ** 9 * s)
            dens.append((B.a / r) ** 6 * s)
    rho = np.linspace(0.0, rho_max, nrho)
    emb = [-sp.c * sp.eps * np.sqrt(rho) for sp in species]
    names = (prefix + ".pt", prefix + ".rho", prefix + ".emb")
    ncol = nt * nt
    write_table2(names[0], [rmin * rmin] * ncol, [rc * rc] * ncol, [step] * ncol, pair)
    write_table2(names[1], [rmin * rmin] * ncol, [rc * rc] * ncol, [step] * ncol, dens)
    rstep = rho_max / (nrho - 1)
    write_table2(names[2], [0.0] * nt, [rho_max] * nt, [rstep] * nt, emb)
    return names


def write_param(path: str, **tok) -> None:
    """IMD parameter file: one ``token value...`` per line."""
    with open(path, "w") as f:
        for k, v in tok.items():
            if isinstance(v, (list, tuple)):
                v = " ".join(str(x) for x in v)
            f.write("%s %s\n" % (k, v))


def write_config(path: str, box: np.ndarray, number, types, mass, x,
                 p=None) -> None:
    """IMD ASCII configuration (format 'A'; number type mass x y z [vx vy vz];
    src/imd_io.c:3369-3489 reads the header).  Velocities are momenta/mass."""
    n = len(number)
    nv = 0 if p is None else 3
    with open(path, "w") as f:
        f.write("#F A 1 1 1 3 %d 0\n" % nv)
        f.write("#C number type mass x y z" + (" vx vy vz\n" if nv else "\n"))
        for lab, v in zip("XYZ", box):
            f.write("#%s %s %s %s\n" % (lab, _fmt(v[0]), _fmt(v[1]), _fmt(v[2])))
        f.write("#E\n")
        for i in range(n):
            row = [str(int(number[i])), str(int(types[i])), _fmt(mass[i])]
            row += [_fmt(v) for v in x[i]]
            if nv:
                row += [_fmt(v) for v in p[i] / mass[i]]
            f.write(" ".join(row) + "\n")


# ---------------------------------------------------------------------------
# crystals
# ---------------------------------------------------------------------------

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5],
                      [0.0, 0.5, 0.5]])


def fcc(n1: int, n2: int, n3: int, a0: float) -> tuple[np.ndarray, np.ndarray]:
    """fcc crystal of n1 x n2 x n3 cubic cells; returns (positions, box rows).
    Atoms sit at (cell + basis + 1/4) a0 so none lies on a cell face."""
    g = np.stack(np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3),
                             indexing="ij"), -1).reshape(-1, 1, 3)
    x = ((g + FCC_BASIS[None] + 0.25) * a0).reshape(-1, 3)
    box = np.diag([n1 * a0, n2 * a0, n3 * a0]).astype(np.float64)
    return x.astype(np.float64), box


def maxwell_momenta(mass: np.ndarray, kT: float, seed: int) -> np.ndarray:
    """Gaussian momenta with variance m kT per component, centre-of-mass
    momentum removed (the distribution IMD's maxwell draws,
    src/imd_maxwell.c:45-297)."""
    rng = np.random.default_rng(seed)
    p = rng.standard_normal((len(mass), 3)) * np.sqrt(kT * mass)[:, None]
    p -= p.mean(axis=0, keepdims=True)
    return p


@dataclass
class System:
    """A single simulation cell in host memory (atom-major arrays)."""
    box: np.ndarray              # (3,3) rows = box vectors
    x: np.ndarray                # (n,3)
    p: np.ndarray                # (n,3)
    types: np.ndarray            # (n,) int32
    mass: np.ndarray             # (n,)
    number: np.ndarray           # (n,) int32
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.x)


def lj_fcc_system(ncell: int = 10, density: float = 0.8442, kT: float = 0.72,
                  seed: int = 1) -> System:
    """Lennard-Jones fcc crystal, reduced units (mass 1)."""
    a0 = (4.0 / density) ** (1.0 / 3.0)
    x, box = fcc(ncell, ncell, ncell, a0)
    n = len(x)
    mass = np.ones(n)
    p = maxwell_momenta(mass, kT, seed)
    return System(box, x, p, np.zeros(n, np.int32), mass,
                  np.arange(n, dtype=np.int32), {"a0": a0})


def eam_fcc_system(ncell: int = 40, a0: float = 3.615, T: float = 300.0,
                   seed: int = 2, species=(CU,), fractions=None,
                   type_seed: int = 3) -> System:
    """Sutton-Chen fcc crystal with Maxwell momenta at temperature T (K).
    With two species, types are assigned by `fractions` uniformly at random."""
    x, box = fcc(ncell, ncell, ncell, a0)
    n = len(x)
    if len(species) == 1:
        types = np.zeros(n, np.int32)
    else:
        rng = np.random.default_rng(type_seed)
        types = (rng.random(n) < (fractions or [0.5])[0]).astype(np.int32)
        types = 1 - types
    mass = np.array([species[t].mass for t in types], np.float64)
    p = maxwell_momenta(mass, KB_EV * T, seed)
    return System(box, x, p, types, mass, np.arange(n, dtype=np.int32), {"a0": a0})


def defect_cell(rng, a0: float = 3.615, nmin: int = 500, nmax: int = 20000,
                nlim=(3, 18), species=CU, strain: float = 0.02, noise: float = 0.05,
                dumbbell: float = 0.3, min_sep: float = 1.8) -> System:
    """One cell of the batched-relaxation workload: an n1 x n2 x n3 fcc cell
    (n_i in nlim) whose atom count follows a log-uniform target in
    [nmin, nmax]; 1-4 defects, each a vacancy or a <100> dumbbell
    interstitial (the site's atom replaced by two atoms at +-dumbbell*a0
    along a random cube axis) at uniformly chosen sites; a homogeneous
    deformation I + e with every component of e uniform in +-strain (a
    triclinic box); Gaussian position noise of `noise` Angstrom.

    Sites are drawn again when two defects would overlap: when an atom of a
    dumbbell comes closer than `min_sep` to another atom (two dumbbells on
    neighbouring sites can put two atoms 1 A apart, where the pair table is
    below its first point and CG cannot move them apart)."""
    lo, hi = nlim
    while True:
        target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        n1, n2 = (int(v) for v in rng.integers(lo, hi + 1, size=2))
        n3 = int(round(target / (4.0 * n1 * n2)))
        if lo <= n3 <= hi:
            break
    x0, box0 = fcc(n1, n2, n3, a0)
    ndef = int(rng.integers(1, 5))
    while True:
        x = x0.copy()
        sites = rng.choice(len(x), size=ndef, replace=False)
        keep = np.ones(len(x), bool)
        extra, moved = [], []
        for site in sites:
            if rng.integers(0, 2) == 0:
                keep[site] = False
            else:
                d = np.zeros(3)
                d[int(rng.integers(0, 3))] = dumbbell * a0
                extra.append(x[site] + d)
                x[site] = x[site] - d
                moved.append(int(site))
        x = np.concatenate([x[keep], np.array(extra).reshape(-1, 3)])
        if not extra:
            break
        # dumbbell atoms: the displaced site atoms (kept) and the added ones
        new_index = np.cumsum(keep) - 1
        probe = np.concatenate([new_index[moved], len(x) - len(extra) + np.arange(len(extra))])
        L = np.diag(box0)
        ok = True
        for i in probe:
            d = x - x[i]
            d -= L * np.round(d / L)
            r2 = np.einsum("ij,ij->i", d, d)
            r2[i] = np.inf
            if r2.min() < min_sep * min_sep:
                ok = False
                break
        if ok:
            break
    F = np.eye(3) + rng.uniform(-strain, strain, size=(3, 3))
    x = x @ F.T
    box = box0 @ F.T
    x = x + noise * rng.standard_normal(x.shape)
    n = len(x)
    return System(box, x, np.zeros((n, 3)), np.zeros(n, np.int32),
                  np.full(n, species.mass), np.arange(n, dtype=np.int32),
                  {"dims": (n1, n2, n3), "defects": ndef})


def defect_batch(ncells: int = 512, seed: int = 4, **kw) -> list:
    """The batched CG workload: `ncells` independent defect cells (seeded)."""
    rng = np.random.default_rng(seed)
    return [defect_cell(rng, **kw) for _ in range(ncells)]
