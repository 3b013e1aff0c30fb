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
    # moves the CG's charges by up to a few 1e-6 (bars of the
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


def read_bonds(path):
    """One frame of a fix reax/c/bonds file: {tag: (type, partner tags, bond
    orders, abo, nlp, q)} and the header's max bond count."""
    rows, most = {}, None
    for line in open(path):
        if line.startswith("# Max number of bonds"):
            most = int(line.split()[7])
        elif not line.startswith("#"):
            w = line.split()
            tag, typ, nb = int(w[0]), int(w[1]), int(w[2])
            ids = [int(v) for v in w[3:3 + nb]]
            bo = [float(v) for v in w[4 + nb:4 + 2 * nb]]
            abo, nlp, q = (float(v) for v in w[4 + 2 * nb:7 + 2 * nb])
            rows[tag] = (typ, ids, bo, abo, nlp, q)
    return rows, most


def test_bond_table_matches_oracle(ffield):
    """rg_bond_table (fix reax/c/bonds, FindBond with bg_cut = 0.3) against
    the oracle's corrected bond orders, total bond order and lone pairs."""
    s = systems.water_box(300, seed=4)
    g = ReaxGPU(ffield)
    g.set_system(s)
    g.qeq()
    g.compute()
    nb, tg, bo, tot, nlp = g.bond_table(0.3, 12)
    o = Oracle(ffield)
    o.set_system(s.box, s.x, s.types(g.elements), s.tag, None, s.v)
    o.qeq()
    o.compute()
    ti, tj, _, obo = o.bond_list()
    at = o.atom_terms()
    idx = {t: k for k, t in enumerate(s.tag)}
    for a in range(s.n):
        sel = (ti == s.tag[a]) & (obo[:, 0] > 0.3)
        want = sorted(zip(tj[sel], obo[sel, 0]))
        got = sorted(zip(tg[a, :nb[a]], bo[a, :nb[a]]))
        assert [w[0] for w in want] == [x[0] for x in got]
        assert np.allclose([w[1] for w in want], [x[1] for x in got], rtol=1e-9, atol=1e-12)
        k = idx[s.tag[a]]
        assert abs(tot[a] - obo[ti == s.tag[a], 0].sum()) < 1e-9
        assert abs(nlp[a] - at[k, 6]) < 1e-9
    assert nb.max() >= 2


def test_deck_bonds_file(tmp_path, ffield):
    """fix reax/c/bonds in a deck writes the reference's file format, one
    frame per Nevery steps, with the library's bond table."""
    s = systems.water_box(150, seed=2)
    data = tmp_path / "sys.data"
    els = systems.write_lammps_data(s, str(data), ["H", "O"])
    deck = [
        "units real", "atom_style charge", "boundary p p p", f"read_data {data}",
        "pair_style reax/c/sunway NULL", f"pair_coeff * * {ffield} {' '.join(els)}",
        "fix 1 all nve/sunway", "fix 2 all qeq/reax/sunway 1 0.0 10.0 1.0e-6 reax/c",
        "fix 3 all reax/c/bonds 5 bonds.reaxc", "timestep 0.25", "run 10",
        f"write_dump all custom out.dump {COLS}",
    ]
    (tmp_path / "in.deck").write_text("\n".join(deck) + "\n")
    r = subprocess.run([B.build_host(), "in.deck"], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    text = (tmp_path / "bonds.reaxc").read_text()
    assert [int(l.split()[2]) for l in text.splitlines() if l.startswith("# Timestep")] == [0, 5, 10]
    last = text[text.rindex("# Timestep"):]
    (tmp_path / "last.reaxc").write_text(last)
    rows, most = read_bonds(str(tmp_path / "last.reaxc"))
    assert len(rows) == s.n and most == max(len(v[1]) for v in rows.values())
    meta, st = read_dump(str(tmp_path / "out.dump"))
    # the last frame is the final state: its charges are the dump's
    for t, qv in zip(st["tag"], st["q"]):
        assert abs(rows[t][5] - qv) < 1e-3
    # every bond listed from both ends with the same order (to the printed 3 decimals)
    for t, (_, ids, bo, _, _, _) in rows.items():
        for j, b in zip(ids, bo):
            back = rows[j][1].index(t)
            assert abs(rows[j][2][back] - b) < 1.5e-3
        assert all(b > 0.3 - 5e-4 for b in bo)
    # O has two H partners in intact water
    types = {t: v[0] for t, v in rows.items()}
    o_type = els.index("O") + 1
    assert np.mean([len(v[1]) == 2 for t, v in rows.items() if types[t] == o_type]) > 0.9


def test_deck_species(tmp_path, ffield):
    """fix reax/c/species in a deck (reference species and position file
    formats): at the last output step its molecules and species equal the
    connected components of the library's bond table (orders above 0.3)
    for the deck's final positions, computed here independently."""
    s = systems.mixture(scale=0.0005, seed=3)
    data = tmp_path / "mix.data"
    els = systems.write_lammps_data(s, str(data), ["C", "H", "O", "N"])
    deck = [
        "units real", "atom_style charge", "boundary p p p", f"read_data {data}",
        "pair_style reax/c/sunway NULL", f"pair_coeff * * {ffield} {' '.join(els)}",
        "fix 1 all nve/sunway", "fix 2 all qeq/reax/sunway 1 0.0 10.0 1.0e-6 reax/c",
        "fix 3 all reax/c/species 1 1 5 species.out position 5 pos.out",
        "timestep 0.25", "run 10", f"write_dump all custom out.dump {COLS}",
    ]
    (tmp_path / "in.deck").write_text("\n".join(deck) + "\n")
    r = subprocess.run([B.build_host(), "in.deck"], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    _, st = read_dump(str(tmp_path / "out.dump"))
    # independent: union-find over the bond table of the final positions
    g = ReaxGPU(ffield)
    order = np.argsort(s.tag)
    g.set_box(s.box)
    g.set_atoms(st["x"], s.types(g.elements)[order], st["tag"], st["q"], st["v"])
    g.compute()
    nb, tg, bo, _, _ = g.bond_table(0.10, 24)
    idx = {t: k for k, t in enumerate(st["tag"])}
    parent = list(range(s.n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for a in range(s.n):
        for k in range(nb[a]):
            if bo[a, k] > 0.3:
                parent[find(a)] = find(idx[tg[a, k]])
    elem = np.array(s.elem)[order]
    comps = {}
    for a in range(s.n):
        comps.setdefault(find(a), []).append(a)
    want = {}
    for atoms in comps.values():
        cnt = [sum(1 for a in atoms if elem[a] == e) for e in els]
        f = "".join(e + (str(c) if c != 1 else "") for e, c in zip(els, cnt) if c)
        want[f] = want.get(f, 0) + 1
    lines = (tmp_path / "species.out").read_text().splitlines()
    assert len(lines) == 4                                  # steps 5 and 10
    assert lines[0].split()[:4] == ["#", "Timestep", "No_Moles", "No_Specs"]
    names = lines[2].split()[4:]
    vals = lines[3].split()
    assert int(vals[0]) == 10
    assert int(vals[1]) == len(comps) and int(vals[2]) == len(want)
    assert dict(zip(names, map(int, vals[3:]))) == want
    pos = (tmp_path / "pos.out").read_text().split("#\n")
    frame = [l.split() for l in pos[-2].splitlines()[2:]]
    assert pos[-2].startswith("Timestep 10 NMole")
    assert len(frame) == len(comps)
    assert sum(int(w[1]) for w in frame) == s.n
    assert all(0.0 <= float(x) < 1.0 for w in frame for x in w[4:7])


def test_deck_thermo_pressure(tmp_path, ffield):
    """The deck's thermo pressure is LAMMPS's compute pressure in real
    units: (2 KE + W_xx + W_yy + W_zz) / 3V * nktv2p with the pair virial
    (rg_get_virial), and its temperature 2 KE / ((3N - 3) k_B)."""
    s = systems.water_box(300, seed=3)
    (meta, st), out = run_deck(tmp_path, s, 0)
    head = [l.split() for l in out.splitlines() if l.split()[:2] == ["Step", "Temp"]]
    row = [l.split() for l in out.splitlines() if l.split() and l.split()[0] == "0"][0]
    cols = dict(zip(head[0], row))
    ke, temp, press = float(cols["KinEng"]), float(cols["Temp"]), float(cols["Press"])
    assert abs(temp - 2 * ke / ((3 * s.n - 3) * 0.0019872067)) < 1e-6 * temp
    g = ReaxGPU(ffield)
    g.set_system(s)
    g.qeq()
    g.compute(vflag=1)
    w = g.virial()[0]
    vol = float(np.prod(s.box))
    want = (2 * ke + w[0] + w[1] + w[2]) / (3 * vol) * 68568.415
    # charges of the deck's and this handle's QEq agree to ~1e-6 e
    assert abs(press - want) < 1e-4 * (abs(want) + 2 * ke / (3 * vol) * 68568.415)
