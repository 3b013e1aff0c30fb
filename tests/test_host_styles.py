"""C++ host styles (sw_reaxff_gb300/host): pair reax/c, fix qeq/reax and fix
nve over the C ABI, with the reference's argument lists and error messages
(PairReaxCSunway::settings/coeff/init_style, pair_reaxc_sunway.cpp:202-424;
FixQEqReaxSunway constructor, fix_qeq_reax_sunway.cpp:64-90; FixNVESunway
constructor, fix_nve_sunway.cpp:29-36; FixReaxCBondsSunway constructor,
fix_reaxc_bonds_sunway.cpp:45-60, 125; FixReaxCSpeciesSunway constructor,
fix_reaxc_species_sunway.cpp:49-238), driven by the reax_md deck
interpreter.  Every deck here fails before the first device call, so these
run without a GPU; the device runs are in test_gpu_host_styles.py."""
import os
import subprocess

import pytest

from sw_reaxff_gb300 import build as B
from sw_reaxff_gb300 import systems
from sw_reaxff_gb300.api import DEFAULT_FFIELD, ffield_elements


@pytest.fixture(scope="module")
def reax_md():
    return B.build_host()


@pytest.fixture(scope="module")
def datafile(tmp_path_factory):
    p = tmp_path_factory.mktemp("deck") / "water.data"
    systems.write_lammps_data(systems.water_box(4, seed=1), str(p), ["H", "O"])
    return str(p)


def run_deck(reax_md, tmp_path, lines):
    deck = tmp_path / "in.deck"
    deck.write_text("\n".join(lines) + "\n")
    r = subprocess.run([reax_md, str(deck)], capture_output=True, text=True, timeout=60,
                       cwd=str(tmp_path))
    return r.returncode, r.stdout + r.stderr


def head(datafile):
    return ["units real", "atom_style charge", f"read_data {datafile}"]


PAIR = f"pair_coeff * * {DEFAULT_FFIELD} H O"
QEQ = "fix 2 all qeq/reax/sunway 1 0.0 10.0 1.0e-6 reax/c"

CASES = {
    "no_control": (["pair_style reax/c/sunway"], "Illegal pair_style command"),
    "bad_checkqeq": (["pair_style reax/c NULL checkqeq maybe"], "Illegal pair_style reax/c command"),
    "odd_keywords": (["pair_style reax/c NULL enobonds"], "Illegal pair_style reax/c command"),
    "neg_safezone": (["pair_style reax/c NULL safezone -1"],
                     "Illegal pair_style reax/c safezone command"),
    "neg_mincap": (["pair_style reax/c NULL mincap -3"], "Illegal pair_style reax/c mincap command"),
    "coeff_count": (["pair_style reax/c NULL", f"pair_coeff * * {DEFAULT_FFIELD} H"],
                    "Incorrect args for pair coefficients"),
    "coeff_ij": (["pair_style reax/c NULL", f"pair_coeff 1 1 {DEFAULT_FFIELD} H O"],
                 "Incorrect args for pair coefficients"),
    "bad_element": (["pair_style reax/c NULL", f"pair_coeff * * {DEFAULT_FFIELD} H Xx"],
                    "Non-existent ReaxFF type"),
    "all_null": (["pair_style reax/c NULL", f"pair_coeff * * {DEFAULT_FFIELD} NULL NULL"],
                 "Incorrect args for pair coefficients"),
    "no_ffield": (["pair_style reax/c NULL", "pair_coeff * * missing.reax H O"],
                  "Cannot open ReaxFF potential file missing.reax"),
    "qeq_args": (["pair_style reax/c NULL", PAIR, "fix 2 all qeq/reax 1 0.0 10.0"],
                 "Illegal fix qeq/reax command"),
    "qeq_nevery": (["pair_style reax/c NULL", PAIR, "fix 2 all qeq/reax 0 0.0 10.0 1e-6 reax/c"],
                   "Illegal fix qeq/reax command"),
    "qeq_number": (["pair_style reax/c NULL", PAIR, "fix 2 all qeq/reax 1 0.0 ten 1e-6 reax/c"],
                   "Expected floating point parameter instead of ten"),
    "qeq_dual_typo": (["pair_style reax/c NULL", PAIR,
                       "fix 2 all qeq/reax 1 0.0 10.0 1e-6 reax/c duel"],
                      "Illegal fix qeq/reax command"),
    "nve_args": (["pair_style reax/c NULL", PAIR, "fix 1 all"], "Illegal fix command"),
    "qeq_required": (["pair_style reax/c NULL", PAIR, "fix 1 all nve/sunway", "run 1"],
                     "Pair reax/c requires use of fix qeq/reax"),
    "qeq_taper": (["pair_style reax/c NULL", PAIR, "fix 2 all qeq/reax 1 0.0 -10.0 1e-6 reax/c",
                   "run 1"], "Fix qeq/reax has negative upper Taper radius cutoff"),
    "bonds_args": (["pair_style reax/c NULL", PAIR, "fix 3 all reax/c/bonds 5"],
                   "Illegal fix reax/c/bonds command"),
    "bonds_nevery": (["pair_style reax/c NULL", PAIR, "fix 3 all reax/c/bonds 0 bonds.out"],
                     "Illegal fix reax/c/bonds command"),
    "bonds_no_pair": (["fix 3 all reax/c/bonds 5 bonds.out"],
                      "Cannot use fix reax/c/bonds without pair_style reax/c"),
    "species_args": (["pair_style reax/c NULL", PAIR, "fix 4 all reax/c/species 1 1"],
                     "Illegal fix reax/c/species command"),
    "species_freq": (["pair_style reax/c NULL", PAIR, "fix 4 all reax/c/species 2 3 5 sp.out"],
                     "Illegal fix reax/c/species command"),
    "species_cutoff": (["pair_style reax/c NULL", PAIR,
                        "fix 4 all reax/c/species 1 1 1 sp.out cutoff 1 5 0.3"],
                       "Illegal fix reax/c/species command"),
    "species_pos": (["pair_style reax/c NULL", PAIR,
                     "fix 4 all reax/c/species 1 1 10 sp.out position 5 pos.out"],
                    "Illegal fix reax/c/species command"),
    "species_gz": (["pair_style reax/c NULL", PAIR, "fix 4 all reax/c/species 1 1 1 sp.gz"],
                   "Cannot open gzipped file"),
    "unknown": (["pair_style reax/c NULL", "compute 1 all pe"], "Unknown command"),
    "units": (["pair_style reax/c NULL"], "requires units real"),
}


@pytest.mark.parametrize("case", list(CASES))
def test_deck_errors(reax_md, datafile, tmp_path, case):
    lines, msg = CASES[case]
    deck = head(datafile) + lines
    if case == "units":
        deck = ["units metal"] + deck[1:]
    rc, out = run_deck(reax_md, tmp_path, deck)
    assert rc == 1, out
    assert out.startswith("ERROR: ") and msg in out, out


def test_read_data_errors(reax_md, tmp_path):
    bad = tmp_path / "bad.data"
    bad.write_text("title\n\n3 atoms\n1 atom types\n0 10 xlo xhi\n0 10 ylo yhi\n"
                   "0 10 zlo zhi\n\nAtoms\n\n1 1 0 1 1 1\n2 1 0 2 2 2\n")
    rc, out = run_deck(reax_md, tmp_path, ["units real", f"read_data {bad}"])
    assert rc == 1 and "Unexpected end of data file" in out, out
    rc, out = run_deck(reax_md, tmp_path, ["units real", "read_data nowhere.data"])
    assert rc == 1 and "Cannot open file nowhere.data" in out, out


def test_ffield_elements_host_only():
    # pair_coeff maps LAMMPS types to elements without a device
    assert ffield_elements() == ["C", "H", "O", "N"]
    with pytest.raises(Exception):
        ffield_elements(os.path.join(os.path.dirname(DEFAULT_FFIELD), "nope.reax"))
