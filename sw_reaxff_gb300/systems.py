"""Seeded synthetic molecular systems for the ReaxFF force step.

The reference ships only a TATB crystal deck; the workloads measured here are
seeded synthetic liquids with the molecule mix, density and temperature of
each workload (2,000-molecule water box; 1,048,576-atom H2O/CH4/C2H6/NH3
mixture; small random packs of H2O/CH4/NH3/CO2/C2H6).  Molecules sit on a
jittered FCC lattice with uniformly random orientations; orientations that
put two atoms of different molecules closer than ``min_dist`` are redrawn.

Units are LAMMPS ``real``: Angstrom, g/mol, fs, kcal/mol.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import os
import re

import numpy as np

AVOGADRO = 6.0221367e23
KB_KCAL = 0.0019872067          # kcal/mol/K
MVV2E = 48.88821291 ** 2        # (g/mol) (A/fs)^2 -> kcal/mol

# Element masses used for densities and velocities (matching ffield.reax).
MASS = {"C": 12.0, "H": 1.008, "O": 15.999, "N": 14.0}


def _water():
    r, ang = 0.9572, math.radians(104.52)
    return ["O", "H", "H"], np.array([
        [0.0, 0.0, 0.0],
        [r * math.sin(ang / 2), r * math.cos(ang / 2), 0.0],
        [-r * math.sin(ang / 2), r * math.cos(ang / 2), 0.0]])


def _methane():
    r = 1.09 / math.sqrt(3.0)
    return ["C", "H", "H", "H", "H"], np.array([
        [0, 0, 0], [r, r, r], [r, -r, -r], [-r, r, -r], [-r, -r, r]], float)


def _ammonia():
    r, hnh = 1.012, math.radians(106.7)
    # three H on a cone around z
    s = 2 * math.sin(hnh / 2) / math.sqrt(3.0)        # sin(cone angle)
    c = math.sqrt(max(0.0, 1 - s * s))
    pos = [[0.0, 0.0, 0.0]]
    for k in range(3):
        phi = 2 * math.pi * k / 3
        pos.append([r * s * math.cos(phi), r * s * math.sin(phi), -r * c])
    return ["N", "H", "H", "H"], np.array(pos)


def _ethane():
    rcc, rch = 1.54, 1.09
    th = math.radians(180 - 109.47)
    pos = [[0, 0, -rcc / 2], [0, 0, rcc / 2]]
    for k in range(3):                       # staggered
        phi = 2 * math.pi * k / 3
        pos.append([rch * math.sin(th) * math.cos(phi),
                    rch * math.sin(th) * math.sin(phi),
                    -rcc / 2 - rch * math.cos(th)])
    for k in range(3):
        phi = 2 * math.pi * k / 3 + math.pi / 3
        pos.append([rch * math.sin(th) * math.cos(phi),
                    rch * math.sin(th) * math.sin(phi),
                    rcc / 2 + rch * math.cos(th)])
    return ["C", "C", "H", "H", "H", "H", "H", "H"], np.array(pos)


def _co2():
    r = 1.16
    return ["C", "O", "O"], np.array([[0, 0, 0], [0, 0, r], [0, 0, -r]], float)


MOLECULES = {"H2O": _water(), "CH4": _methane(), "NH3": _ammonia(),
             "C2H6": _ethane(), "CO2": _co2()}


@dataclass
class System:
    """A periodic box of atoms: orthogonal (positions in [0, L)), or
    triclinic with tilt = (xy, xz, yz) (edge vectors (lx,0,0), (xy,ly,0),
    (xz,yz,lz), LAMMPS's restricted form)."""
    box: np.ndarray            # (3,) edge lengths lx, ly, lz
    x: np.ndarray              # (n, 3) float64
    elem: list                 # element symbol per atom
    tag: np.ndarray            # (n,) int32, 1-based
    v: np.ndarray              # (n, 3) float64, A/fs
    mol: np.ndarray            # (n,) molecule index
    meta: dict = field(default_factory=dict)
    tilt: np.ndarray = None    # (3,) xy, xz, yz or None (orthogonal)

    @property
    def triclinic(self) -> bool:
        return self.tilt is not None and bool(np.any(np.asarray(self.tilt) != 0.0))

    @property
    def n(self) -> int:
        return self.x.shape[0]

    def types(self, element_order) -> np.ndarray:
        """ffield type index per atom given the ffield's element order."""
        idx = {e.upper(): i for i, e in enumerate(element_order)}
        return np.array([idx[e.upper()] for e in self.elem], dtype=np.int32)

    def masses(self) -> np.ndarray:
        return np.array([MASS[e] for e in self.elem])


def _random_rotations(rng, k):
    """k uniform random rotation matrices (via unit quaternions)."""
    q = rng.normal(size=(k, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def _cell_table(x, box, cw_min):
    nc = np.maximum((box // cw_min).astype(int), 1)
    cw = box / nc
    ci = np.minimum((x // cw).astype(int), nc - 1)
    cid = (ci[:, 2] * nc[1] + ci[:, 1]) * nc[0] + ci[:, 0]
    order = np.argsort(cid, kind="stable")
    cs = cid[order]
    ncell = int(nc.prod())
    start = np.searchsorted(cs, np.arange(ncell), "left")
    end = np.searchsorted(cs, np.arange(ncell), "right")
    M = int((end - start).max()) if len(x) else 1
    table = np.full((ncell, max(M, 1)), -1, dtype=np.int64)
    rank = np.arange(len(x)) - start[cs]
    table[cs, rank] = order
    return nc, ci, table


def _min_contact(xq, molq, x, mol, box, dmin, table=None):
    """Per query point: the smallest periodic distance to an atom of x that
    belongs to another molecule, when below dmin (else inf)."""
    nc, ci, tab = table if table is not None else _cell_table(x, box, dmin)
    out = np.full(len(xq), np.inf)
    cw = box / nc
    cq = np.minimum((xq // cw).astype(int), nc - 1) % nc
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                nb = (cq + np.array([dx, dy, dz])) % nc
                nid = (nb[:, 2] * nc[1] + nb[:, 1]) * nc[0] + nb[:, 0]
                cand = tab[nid]
                valid = cand >= 0
                cj = np.where(valid, cand, 0)
                d = x[cj] - xq[:, None, :]
                d -= box * np.round(d / box)
                r2 = (d * d).sum(-1)
                r2 = np.where(valid & (mol[cj] != molq[:, None]), r2, np.inf)
                out = np.minimum(out, np.sqrt(r2.min(1)))
    return out


def _fcc_sites(nmol, box, rng):
    """nmol random sites of the smallest FCC lattice with >= nmol points."""
    m = 1
    while 4 * m ** 3 < nmol:
        m += 1
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m),
                             indexing="ij"), -1).reshape(-1, 3).astype(float)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pts = (g[:, None, :] + basis[None]).reshape(-1, 3) + 0.25
    pts = pts[rng.permutation(len(pts))[:nmol]]
    return pts * (box / m)


def pack_molecules(counts: dict, density: float, seed: int, *,
                   temperature: float = 300.0, jitter: float = 0.2,
                   min_dist: float = 1.5, max_redraw: int = 200,
                   atom_jitter: float = 0.02, box=None) -> System:
    """Place molecules (counts: name -> number) in a cubic periodic box at
    ``density`` g/cm^3 on a jittered FCC lattice with random orientations;
    molecules with an intermolecular contact closer than ``min_dist`` get
    new orientations until none is left (or ``max_redraw`` rounds)."""
    rng = np.random.default_rng(seed)
    names = []
    for name, k in counts.items():
        names += [name] * int(k)
    names = np.array(names)
    rng.shuffle(names)
    nmol = len(names)
    mass_total = sum(sum(MASS[e] for e in MOLECULES[nm][0]) * int(k)
                     for nm, k in counts.items())
    if box is None:
        vol = mass_total / AVOGADRO / density * 1e24     # A^3
        L = vol ** (1.0 / 3.0)
        box = np.array([L, L, L])
    box = np.asarray(box, float)
    sites = _fcc_sites(nmol, box, rng)
    centers = sites + rng.uniform(-jitter, jitter, size=sites.shape)
    tries = np.zeros(nmol, dtype=int)
    tmpl_e, tmpl_x, mol_of = [], [], []
    for k, nm in enumerate(names):
        e, xyz = MOLECULES[nm]
        tmpl_e += e
        tmpl_x.append(xyz - xyz.mean(0))
        mol_of += [k] * len(e)
    mol_of = np.array(mol_of)
    local = np.concatenate(tmpl_x)
    # small per-atom distortion: no molecule sits exactly on a symmetric
    # (e.g. linear CO2) geometry, where angle derivatives are singular
    local = local + rng.normal(scale=atom_jitter, size=local.shape)
    rot = _random_rotations(rng, nmol)
    x = (np.einsum("aij,aj->ai", rot[mol_of], local) + centers[mol_of]) % box
    atoms_of = np.split(np.arange(len(x)), np.cumsum(np.bincount(mol_of))[:-1])
    check = np.arange(len(x))
    K = 8
    for it in range(max_redraw):
        tab = _cell_table(x, box, min_dist)
        close = _min_contact(x[check], mol_of[check], x, mol_of, box, min_dist, tab) < min_dist
        bad = np.unique(mol_of[check[close]])
        if len(bad) == 0:
            break
        # best of K new placements (orientation + small move off the site),
        # scored by the closest contact with the current configuration
        tries[bad] += 1
        sel = np.concatenate([atoms_of[b] for b in bad])
        msel = mol_of[sel]
        best = np.full(len(bad), -1.0)
        best_x = x[sel].copy()
        pos_in_bad = np.searchsorted(bad, msel)
        for _ in range(K):
            r = _random_rotations(rng, len(bad))
            amp = np.minimum(jitter + 0.05 * tries[bad], 0.8)[:, None]
            c = sites[bad] + rng.uniform(-1, 1, size=(len(bad), 3)) * amp
            xc = (np.einsum("aij,aj->ai", r[pos_in_bad], local[sel]) + c[pos_in_bad]) % box
            dmin_atom = _min_contact(xc, msel, x, mol_of, box, 3.0, tab)
            dmin_mol = np.full(len(bad), np.inf)
            np.minimum.at(dmin_mol, pos_in_bad, dmin_atom)
            take = dmin_mol > best
            best = np.where(take, dmin_mol, best)
            ta = take[pos_in_bad]
            best_x[ta] = xc[ta]
        x[sel] = best_x
        check = sel
    n = x.shape[0]
    masses = np.array([MASS[e] for e in tmpl_e])
    sig = np.sqrt(KB_KCAL * temperature / (masses * MVV2E))
    v = rng.normal(size=(n, 3)) * sig[:, None]
    p = (v * masses[:, None]).sum(0) / masses.sum()
    v -= p
    x = np.where(x >= box, x - box, x)
    return System(box=box, x=np.ascontiguousarray(x), elem=list(tmpl_e),
                  tag=np.arange(1, n + 1, dtype=np.int32),
                  v=np.ascontiguousarray(v), mol=mol_of,
                  meta={"counts": dict(counts), "density": density,
                        "seed": seed, "temperature": temperature})


def water_box(n_molecules: int = 2000, density: float = 1.0,
              seed: int = 2024) -> System:
    """Liquid water box: 2,000 H2O at 1.0 g/cm^3 is the 6,000-atom case."""
    return pack_molecules({"H2O": n_molecules}, density, seed)


# 1,048,576 atoms exactly: 3*116511 + 5*46603 + 8*46603 + 4*23301
MIXTURE_1M = {"H2O": 116511, "CH4": 46603, "C2H6": 46603, "NH3": 23301}


def mixture(scale: float = 1.0, density: float = 0.8,
            seed: int = 7) -> System:
    """H2O/CH4/C2H6/NH3 mixture, mole fractions 0.5/0.2/0.2/0.1.
    scale=1 gives the 1,048,576-atom system; smaller scales keep the mix."""
    counts = {k: max(1, int(round(v * scale))) for k, v in MIXTURE_1M.items()}
    return pack_molecules(counts, density, seed)


def small_pack(n_atoms_target: int, density: float, seed: int) -> System:
    """Random pack of H2O/CH4/NH3/CO2/C2H6 of about n_atoms_target atoms
    (one system of the batched workload)."""
    rng = np.random.default_rng(seed)
    kinds = ["H2O", "CH4", "NH3", "CO2", "C2H6"]
    counts = {k: 0 for k in kinds}
    n = 0
    while n < n_atoms_target:
        k = kinds[rng.integers(len(kinds))]
        counts[k] += 1
        n += len(MOLECULES[k][0])
    counts = {k: v for k, v in counts.items() if v}
    return pack_molecules(counts, density, seed + 1)


_NUM = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


def _num(tok: str) -> float:
    """The longest numeric prefix of a token, as C's strtod reads it (the
    shipped TATB data file writes "15.1826391451E zlo zhi")."""
    m = _NUM.match(tok)
    if not m:
        raise ValueError(f"not a number: {tok!r}")
    return float(m.group(0))


def read_lammps_data(path: str, elements) -> System:
    """Read a LAMMPS data file of atom_style charge (header counts, box
    bounds, an optional "xy xz yz" tilt line, Masses, Atoms "id type q x y
    z", optional Velocities), the format of the reference's data.tatb.
    LAMMPS type k is elements[k-1].  Positions are taken relative to the
    box origin (xlo, ylo, zlo); velocities default to zero."""
    lines = [ln.split("#")[0].strip() for ln in open(path)]
    n = None
    lo, hi = [0.0] * 3, [0.0] * 3
    tilt = None
    k = 1
    while k < len(lines):
        w = lines[k].split()
        if not w:
            k += 1
            continue
        if w[-1] == "atoms" and len(w) == 2:
            n = int(w[0])
        elif w[-2:] in (["xlo", "xhi"], ["ylo", "yhi"], ["zlo", "zhi"]):
            c = "xyz".index(w[-2][0])
            lo[c], hi[c] = _num(w[0]), _num(w[1])
        elif w[-3:] == ["xy", "xz", "yz"]:
            tilt = np.array([_num(w[0]), _num(w[1]), _num(w[2])])
        elif w[0] in ("Masses", "Atoms", "Velocities"):
            break
        k += 1
    if n is None:
        raise ValueError("data file has no atom count")
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    tag = np.zeros(n, np.int32)
    typ = np.zeros(n, np.int32)
    row = {}
    while k < len(lines):
        sec = lines[k].split()
        k += 1
        if not sec:
            continue
        name = sec[0]
        body = []
        while k < len(lines) and (not lines[k] or lines[k].split()[0][0] in "+-.0123456789"):
            if lines[k]:
                body.append(lines[k].split())
            k += 1
        if name == "Atoms":
            if len(body) != n:
                raise ValueError("Atoms section does not hold every atom")
            for a, w in enumerate(body):
                tag[a], typ[a] = int(w[0]), int(w[1])
                x[a] = [_num(w[3]) - lo[0], _num(w[4]) - lo[1], _num(w[5]) - lo[2]]
                row[tag[a]] = a
        elif name == "Velocities":
            for w in body:
                v[row[int(w[0])]] = [_num(w[1]), _num(w[2]), _num(w[3])]
    box = np.array([hi[c] - lo[c] for c in range(3)])
    elem = [elements[t - 1] for t in typ]
    return System(box=box, x=x, elem=elem, tag=tag, v=v, mol=np.zeros(n, np.int32),
                  meta={"source": os.path.basename(path)}, tilt=tilt)


def replicate(system: System, reps) -> System:
    """The system repeated reps = (na, nb, nc) times along its edge vectors
    (what scaling the TATB deck's box and lattice by S does)."""
    na, nb, nc = reps
    lx, ly, lz = system.box
    xy, xz, yz = system.tilt if system.tilt is not None else (0.0, 0.0, 0.0)
    a, b, c = np.array([lx, 0, 0]), np.array([xy, ly, 0]), np.array([xz, yz, lz])
    xs, els, vs = [], [], []
    for k in range(nc):
        for j in range(nb):
            for i in range(na):
                xs.append(system.x + i * a + j * b + k * c)
                els += list(system.elem)
                vs.append(system.v)
    n = len(els)
    tilt = None if system.tilt is None else np.array([nb * xy, nc * xz, nc * yz])
    return System(box=np.array([na * lx, nb * ly, nc * lz]), x=np.concatenate(xs), elem=els,
                  tag=np.arange(1, n + 1, dtype=np.int32), v=np.concatenate(vs),
                  mol=np.zeros(n, np.int32), meta=dict(system.meta, reps=reps), tilt=tilt)


def write_lammps_data(system: System, path: str, elements=None, q=None) -> list:
    """Write a LAMMPS data file (atom_style charge: Masses, Atoms with
    "id type q x y z", Velocities) of an orthogonal periodic system, the input
    format of the reference's decks (read_data).  LAMMPS type k is
    elements[k-1] (default: the elements present, sorted).  Returns the
    element order for pair_coeff."""
    els = list(elements) if elements is not None else sorted(set(system.elem))
    tidx = {e: k + 1 for k, e in enumerate(els)}
    q = np.zeros(system.n) if q is None else np.asarray(q, np.float64)
    with open(path, "w") as fp:
        fp.write("ReaxFF system written by sw_reaxff_gb300.systems\n\n")
        fp.write(f"{system.n} atoms\n{len(els)} atom types\n\n")
        for c, nm in enumerate(("x", "y", "z")):
            fp.write(f"0.0 {float(system.box[c])!r} {nm}lo {nm}hi\n")
        fp.write("\nMasses\n\n")
        for e in els:
            fp.write(f"{tidx[e]} {float(MASS[e])!r}\n")
        fp.write("\nAtoms # charge\n\n")
        for i in range(system.n):
            x = system.x[i]
            fp.write(f"{int(system.tag[i])} {tidx[system.elem[i]]} {float(q[i])!r} "
                     f"{float(x[0])!r} {float(x[1])!r} {float(x[2])!r}\n")
        fp.write("\nVelocities\n\n")
        for i in range(system.n):
            v = system.v[i]
            fp.write(f"{int(system.tag[i])} {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
    return els
