"""The reference's TATB deck inputs through the C++ deck driver on CPU
(everything before the first device call): in.reaxc.lattice builds its
triclinic crystal with variables, "&" continuations, lattice custom,
region prism, create_box and create_atoms, and the result equals the
shipped data.tatb (read with its "xy xz yz" line) atom for atom; -var S 2
repeats it 2x2x2; the control file's keywords set the cutoffs and an
unknown keyword is an error, as in the reference (Read_Control_File,
reaxc_control_sunway.cpp:33-380)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from sw_reaxff_gb300 import build as B
from sw_reaxff_gb300 import systems
from sw_reaxff_gb300.api import DEFAULT_FFIELD

DATA = os.path.dirname(DEFAULT_FFIELD)
ELEMENTS = ["C", "H", "O", "N"]


@pytest.fixture(scope="module")
def reax_md():
    return B.build_host()


def deck_dir(tmp_path):
    for f in ("in.reaxc.lattice", "control.reax_c.tatb", "ffield.reax", "data.tatb"):
        shutil.copy(os.path.join(DATA, f), tmp_path / f)
    return tmp_path


def run(reax_md, cwd, deck, *args):
    (cwd / "in.test").write_text(deck)
    r = subprocess.run([reax_md, *args, "-in", "in.test"], cwd=str(cwd), capture_output=True,
                       text=True, timeout=60)
    return r.returncode, r.stdout + r.stderr


def read_dump(path):
    rows = np.array([[float(v) for v in l.split()] for l in open(path) if not l.startswith("#")])
    return rows[:, 0].astype(int), rows[:, 1].astype(int), rows[:, 3:6]


def lattice_prefix(d):
    txt = (d / "in.reaxc.lattice").read_text()
    return txt[:txt.index("pair_style")]


def test_lattice_deck_builds_the_data_file_crystal(reax_md, tmp_path):
    d = deck_dir(tmp_path)
    rc, out = run(reax_md, d, lattice_prefix(d) + "write_dump all custom built.dump id type q x y z\n")
    assert rc == 0, out
    tag, typ, x = read_dump(d / "built.dump")
    assert len(tag) == 384 and np.array_equal(tag, np.arange(1, 385))
    s = systems.read_lammps_data(str(d / "data.tatb"), ELEMENTS)
    A = np.array([[s.box[0], 0, 0], [s.tilt[0], s.box[1], 0], [s.tilt[1], s.tilt[2], s.box[2]]])
    Ainv = np.linalg.inv(A)
    tidx = {e: k + 1 for k, e in enumerate(ELEMENTS)}
    data_types = np.array([tidx[e] for e in s.elem])
    used = set()
    for i in range(len(tag)):
        df = (s.x - x[i]) @ Ainv
        df -= np.round(df)
        r = np.linalg.norm(df @ A, axis=1)
        j = int(np.argmin(r))
        assert r[j] < 1e-8 and data_types[j] == typ[i]
        used.add(j)
    assert len(used) == 384


def test_lattice_deck_scaled(reax_md, tmp_path):
    d = deck_dir(tmp_path)
    rc, out = run(reax_md, d, lattice_prefix(d) + "write_dump all custom b.dump id type x y z\n",
                  "-var", "S", "2")
    assert rc == 0, out
    tag, typ, _ = read_dump(d / "b.dump")
    assert len(tag) == 8 * 384 and np.bincount(typ).tolist() == [0] + [768] * 4


def test_read_data_triclinic(reax_md, tmp_path):
    d = deck_dir(tmp_path)
    deck = ("units real\natom_style charge\nread_data data.tatb\n"
            "write_dump all custom r.dump id type q x y z\n")
    rc, out = run(reax_md, d, deck)
    assert rc == 0, out
    tag, typ, x = read_dump(d / "r.dump")
    s = systems.read_lammps_data(str(d / "data.tatb"), ELEMENTS)
    assert np.allclose(x, s.x) and np.array_equal(tag, s.tag)


CONTROL_ERRORS = {
    "unknown": ("nbrhood_cutoff 4.5\nbogus_keyword 1\n", "Unknown parameter bogus_keyword"),
}


def test_control_file_errors(reax_md, tmp_path):
    d = deck_dir(tmp_path)
    (d / "bad.control").write_text(CONTROL_ERRORS["unknown"][0])
    head = "units real\natom_style charge\nread_data data.tatb\n"
    rc, out = run(reax_md, d, head + "pair_style reax/c bad.control\n")
    assert rc == 1 and CONTROL_ERRORS["unknown"][1] in out, out
    rc, out = run(reax_md, d, head + "pair_style reax/c missing.control\n")
    assert rc == 1 and "Cannot open control file missing.control" in out, out
    # the shipped control file and the deck's own pair_style line are accepted
    rc, out = run(reax_md, d, head + "pair_style reax/c control.reax_c.tatb maxfar 512\n"
                  "pair_coeff * * ffield.reax C H O N\n")
    assert rc == 0, out


def test_variable_errors(reax_md, tmp_path):
    rc, out = run(reax_md, tmp_path, "variable a equal 2*(3\nunits real\nvariable b equal ${a}\n")
    assert rc == 1 and "Invalid syntax in variable formula" in out, out
    rc, out = run(reax_md, tmp_path, "units real\nvariable b equal $Q*2\n")
    assert rc == 1 and "Substitution for illegal variable Q" in out, out
