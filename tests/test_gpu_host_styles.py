"""The C++ host styles on the GPU: a LAMMPS deck written with the reference's
style names (pair_style reax/c/sunway, fix qeq/reax/sunway, fix nve/sunway)
run by reax_md gives the forces, charges and energies of the C ABI called
directly and of the CPU oracle, and its NVE trajectory follows rg_run's."""
import subprocess

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300 import build as B

pytestmark = pytest.mark.gpu

COLS = "id type q x y z vx vy vz fx fy fz"


def read_dump(path):
    meta = {}
    rows = []
    for line in open(path):
        if line.startswith("# pvector"):
            meta["pvector"] = np.array([float(v) for v in line.split()[2:]])
        elif line.startswith("# eng_vdwl"):
            w = line.split()
            meta["eng_vdwl"], meta["eng_coul"] = float(w[2]), float(w[4])
        elif not line.startswith("#"):
            rows.append([float(v) for v in line.split()])
    a = np.array(rows)
    return meta, dict(tag=a[:, 0].astype(int), q=a[:, 2], x=a[:, 3:6], v=a[:, 6:9], f=a[:, 9:12])


def run_deck(tmp_path, s, nsteps, dump="out.dump"):
    data = tmp_path / "sys.data"
    els = systems.write_lammps_data(s, str(data), ["H", "O"])
    from sw_reaxff_gb300.api import DEFAULT_FFIELD
    deck = [
        "units real", "atom_style charge", "boundary p p p", f"read_data {data}",
        "pair_style reax/c/sunway NULL checkqeq yes",
        f"pair_coeff * * {DEFAULT_FFIELD} {' '.join(els)}",
        "neighbor 2.5 bin", "neigh_modify every 1 delay 0 check no",
        "fix 1 all nve/sunway",
        "fix 2 all qeq/reax/sunway 1 0.0 10.0 1.0e-6 reax/c",
        "timestep 0.25", "thermo 5", f"run {nsteps}",
        f"write_dump all custom {dump} {COLS}",
    ]
    (tmp_path / "in.deck").write_text("\n".join(deck) + "\n")
    r = subprocess.run([B.build_host(), "in.deck"], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return read_dump(str(tmp_path / dump)), r.stdout


def test_deck_single_point_matches_abi_and_oracle(tmp_path, ffield):
    s = systems.water_box(200, seed=1)
    (meta, st), out = run_deck(tmp_path, s, 0)
    assert "PotEng" in out
    g = ReaxGPU(ffield)
    g.set_system(s)
    qg, _, _ = g.qeq()
    fg, eg = g.compute()
    order = np.argsort(s.tag)
    assert np.array_equal(st["tag"], s.tag[order])
    # same library, same calls: equal up to the order of FP64 atomics, which
    # moves the pipelined CG's charges by up to a few 1e-6 (bars of the
    # batch tests: 1e-5)
    assert np.abs(st["q"] - qg[order]).max() < 1e-5
    assert np.sqrt(((st["f"] - fg[order]) ** 2).sum() / (fg ** 2).sum()) < 1e-5
    assert abs(meta["eng_vdwl"] - eg["eng_vdwl"]) < 1e-5 * abs(eg["eng_vdwl"])
    o = Oracle(ffield)
    o.set_system(s.box, s.x, s.types(g.elements), s.tag, None, s.v)
    qo, _, _ = o.qeq()
    fo, eo = o.compute()
    assert np.abs(st["q"] - qo[order]).max() < 1e-5
    assert np.sqrt(((st["f"] - fo[order]) ** 2).sum() / (fo ** 2).sum()) < 1e-5
    pe = meta["eng_vdwl"] + meta["eng_coul"]
    assert abs(pe - (eo["eng_vdwl"] + eo["eng_coul"])) < 1e-5 * abs(pe)


def test_deck_nve_follows_rg_run(tmp_path, ffield):
    s = systems.water_box(200, seed=5)
    (meta, st), out = run_deck(tmp_path, s, 10)
    g = ReaxGPU(ffield)
    g.set_system(s)
    g.run(10, 0.25)
    x, v, q, f = g.get_atoms()
    order = np.argsort(s.tag)
    L = s.box
    dx = st["x"] - x[order]
    dx -= L * np.round(dx / L)        # either side may have wrapped
    # the CG charges move by up to a few 1e-6 per solve when FP64 atomics
    # reorder; over 10 steps of extrapolated solves that reaches ~1e-5 in
    # the charges, ~1e-7 A in the positions and ~1e-8 A/fs in the velocities
    assert np.abs(dx).max() < 1e-5
    assert np.abs(st["v"] - v[order]).max() < 1e-5
    assert np.abs(st["q"] - q[order]).max() < 5e-5
    lines = [ln for ln in out.splitlines() if ln.strip() and ln.split()[0].isdigit()]
    assert [int(ln.split()[0]) for ln in lines] == [0, 5, 10]
    etot = [float(ln.split()[3]) for ln in lines]
    # NVE: total energy drifts by far less than the kinetic energy
    assert abs(etot[-1] - etot[0]) < 0.05 * abs(float(lines[0].split()[2]))
