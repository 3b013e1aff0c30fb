"""Triclinic cells on the GPU against the oracle: the reference's TATB
crystal (data.tatb, the prism box of its in.reaxc.lattice deck, with the
deck's control file cutoffs: bonds 4.5 A, H-bonds 6.0 A) as shipped (384
atoms; every cell width above the 10 A cutoff needs periodic images of
several lattice indices) and repeated 2x2x2, and a water box described by
a triclinic cell of the same lattice.  Bars as for orthogonal boxes: lists
equal as sets, energies 1e-9 relative and forces 1e-9 relative RMS at the
same charges, charges 1e-5 e; the mixed form at its bars (forces 1e-4
relative RMS, charges 1e-5 e)."""
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import DEFAULT_FFIELD, PREC_MIXED

pytestmark = pytest.mark.gpu

DATA = os.path.join(os.path.dirname(DEFAULT_FFIELD), "data.tatb")
TATB_CTL = dict(bond_cut=4.5, hbond_cut=6.0)       # control.reax_c.tatb
ELEMENTS = ["C", "H", "O", "N"]                      # pair_coeff * * ffield.reax C H O N

E_TERMS = ["e_bond", "e_ovun", "e_lp", "e_ang", "e_pen", "e_coa", "e_hb", "e_tor", "e_con",
           "e_vdW", "e_ele", "e_pol", "eng_vdwl", "eng_coul", "e_pol_phys"]


def tatb(reps=(1, 1, 1)):
    s = systems.read_lammps_data(DATA, ELEMENTS)
    return s if reps == (1, 1, 1) else systems.replicate(s, reps)


def water_tilted():
    s = systems.water_box(200, seed=1)
    lx, ly, _ = s.box
    s.tilt = np.array([lx, -lx, ly])        # b' = a + b, c' = c - a + b
    return s


CASES = {
    "tatb": (lambda: tatb(), TATB_CTL),
    "tatb222": (lambda: tatb((2, 2, 2)), TATB_CTL),
    "water_tilted": (water_tilted, {}),
}


def keyset(ti, tj, im):
    return set(zip(ti.tolist(), tj.tolist(), im.tolist()))


def oracle_for(ffield, s, ctl):
    o = Oracle(ffield, **ctl)
    o.set_system(s.box, s.x, s.types(ELEMENTS), s.tag, None, s.v, tilt=s.tilt)
    return o


@pytest.fixture(scope="module", params=list(CASES))
def run(request, ffield):
    make, ctl = CASES[request.param]
    s = make()
    o = oracle_for(ffield, s, ctl)
    qo = o.qeq()
    fo, eo = o.compute()
    g = ReaxGPU(ffield, **ctl)
    g.set_system(s)
    g.set_atoms(s.x, s.types(g.elements), s.tag, qo[0], s.v)
    fg, eg = g.compute()
    g2 = ReaxGPU(ffield, **ctl)
    g2.set_system(s)
    qg = g2.qeq()
    fg2, _ = g2.compute()
    return dict(s=s, g=g, o=o, qo=qo, fo=fo, eo=eo, fg=fg, eg=eg, qg=qg, fg2=fg2)


def test_lists_equal(run):
    assert keyset(*run["g"].pair_list()) == keyset(*run["o"].far_list())
    gi, gj, gm, _ = run["g"].bond_list()
    oi, oj, om, _ = run["o"].bond_list()
    assert keyset(gi, gj, gm) == keyset(oi, oj, om) and len(oi) > 0
    assert keyset(*run["g"].hbond_list()) == keyset(*run["o"].hbond_list())


def test_energies_and_forces_same_charges(run):
    eo, eg = run["eo"], run["eg"]
    for k in E_TERMS:
        assert abs(eg[k] - eo[k]) <= max(1e-9 * abs(eo[k]), 1e-7), (k, eg[k], eo[k])
    fo, fg = run["fo"], run["fg"]
    assert np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-9


def test_charges_and_chain(run):
    assert np.abs(run["qg"][0] - run["qo"][0]).max() < 1e-5
    fo, fg2 = run["fo"], run["fg2"]
    assert np.sqrt(((fg2 - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-5


def test_mixed_tatb(ffield):
    s = tatb((2, 2, 2))
    o = oracle_for(ffield, s, TATB_CTL)
    qo, _, _ = o.qeq()
    fo, eo = o.compute()
    g = ReaxGPU(ffield, precision=PREC_MIXED, **TATB_CTL)
    g.set_system(s)
    qg, _, _ = g.qeq()
    fg, eg = g.compute()
    assert keyset(*g.pair_list()) == keyset(*o.far_list())
    gi, gj, gm, _ = g.bond_list()
    oi, oj, om, _ = o.bond_list()
    assert keyset(gi, gj, gm) == keyset(oi, oj, om)
    assert np.abs(qg - qo).max() < 1e-5
    assert np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-4
    pe = eo["eng_vdwl"] + eo["eng_coul"]
    assert abs(eg["eng_vdwl"] + eg["eng_coul"] - pe) < 1e-4 * abs(pe)


def test_same_lattice_on_gpu(ffield):
    """Orthogonal water box and its triclinic description: same energies
    and forces at the same charges."""
    s0 = systems.water_box(200, seed=1)
    s1 = water_tilted()
    o = oracle_for(ffield, s0, {})
    q, _, _ = o.qeq()
    out = []
    for s in (s0, s1):
        g = ReaxGPU(ffield)
        g.set_system(s)
        g.set_atoms(s.x, s.types(g.elements), s.tag, q, s.v)
        out.append(g.compute())
    (f0, e0), (f1, e1) = out
    assert np.sqrt(((f1 - f0) ** 2).sum() / (f0 ** 2).sum()) < 1e-9
    for k in E_TERMS:
        assert abs(e1[k] - e0[k]) <= max(1e-9 * abs(e0[k]), 1e-7), k


def test_tatb_deck_end_to_end(ffield, tmp_path):
    """The reference's in.reaxc.lattice deck, unchanged but for an appended
    write_dump, run by reax_md: its single point (-var t 0) equals the
    oracle's on the crystal it builds (control-file cutoffs), and its 10
    NVE steps (dt 0.625 fs) follow rg_run on the same start."""
    import shutil
    import subprocess
    from sw_reaxff_gb300 import build as B
    for f in ("in.reaxc.lattice", "control.reax_c.tatb", "ffield.reax"):
        shutil.copy(os.path.join(os.path.dirname(DEFAULT_FFIELD), f), tmp_path / f)
    deck = (tmp_path / "in.reaxc.lattice").read_text()
    cols = "id type q x y z vx vy vz fx fy fz"
    (tmp_path / "in.deck").write_text(deck + f"\nwrite_dump all custom out.dump {cols}\n")
    exe = B.build_host()

    def run(*args):
        r = subprocess.run([exe, *args, "-in", "in.deck"], cwd=str(tmp_path),
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        rows = np.array([[float(v) for v in l.split()] for l in open(tmp_path / "out.dump")
                         if not l.startswith("#")])
        meta = [l for l in open(tmp_path / "out.dump") if l.startswith("# eng_vdwl")][0].split()
        return rows, float(meta[2]) + float(meta[4])

    rows, pe = run("-var", "t", "0")
    s = tatb()
    # the deck's crystal in tag order: the data file's atoms (same sites)
    x0 = rows[:, 3:6]
    types = rows[:, 1].astype(int) - 1            # LAMMPS types 1..4 = C H O N
    o = Oracle(ffield, **TATB_CTL)
    o.set_system(s.box, x0, types, rows[:, 0].astype(int), None, None, tilt=s.tilt)
    qo, _, _ = o.qeq()
    fo, eo = o.compute()
    assert np.abs(rows[:, 2] - qo).max() < 1e-5
    fd = rows[:, 9:12]
    assert np.sqrt(((fd - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-5
    assert abs(pe - (eo["eng_vdwl"] + eo["eng_coul"])) < 1e-5 * abs(pe)

    rows10, _ = run()
    g = ReaxGPU(ffield, **TATB_CTL)
    sysx = systems.System(box=s.box, x=x0, elem=[ELEMENTS[t] for t in types],
                          tag=rows[:, 0].astype(np.int32), v=np.zeros_like(x0),
                          mol=np.zeros(len(x0), np.int32), tilt=s.tilt)
    g.set_system(sysx)
    g.set_masses(np.array([12.0, 1.008, 15.999, 14.0]))   # the deck's mass commands
    g.run(10, 0.625)
    x, v, q, f = g.get_atoms()
    # positions modulo the lattice (both wrap into the cell)
    A = np.array([[s.box[0], 0, 0], [s.tilt[0], s.box[1], 0], [s.tilt[1], s.tilt[2], s.box[2]]])
    df = (rows10[:, 3:6] - x) @ np.linalg.inv(A)
    df -= np.round(df)
    assert np.abs(df @ A).max() < 1e-6
    assert np.abs(rows10[:, 6:9] - v).max() < 1e-6
