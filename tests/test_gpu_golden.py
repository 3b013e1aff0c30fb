"""The CUDA force step against the golden fixtures of the reference's own
code (same positions and charges): bond and H-bond lists as sets, corrected
bond orders within 1e-10, per-term energies within 1e-9 relative, forces
within 1e-9 relative RMS.  The CUDA QEq against the charges of the
reference's own QEq driver (1e-5 e, the charge bar), and 5 NVE steps
against the fixture's trajectory on the reference's QEq (charges there
within the CG's own stopping error, 5e-5 e)."""
import glob
import os

import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
TERMS = ["e_bond", "e_ovun", "e_lp", "e_ang", "e_pen", "e_coa", "e_hb", "e_tor",
         "e_con", "e_vdW", "e_ele", "e_pol", "eng_vdwl", "eng_coul"]


def keyset(ti, tj, im):
    return set(zip(ti.tolist(), tj.tolist(), im.tolist()))


@pytest.fixture(scope="module", params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def case(request, ffield):
    z = np.load(request.param)
    g = {k: z[k] for k in z.files}
    gpu = ReaxGPU(ffield)
    gpu.set_box(g["box"])
    gpu.set_atoms(g["x"], g["types"], g["tags"], g["q"])
    f, e = gpu.compute(eflag=3, vflag=4)
    return g, gpu, f, e


def test_gpu_atom_tallies_vs_reference(case):
    """Per-atom energy and virial against the reference's ev_tally_full:
    1e-9 relative RMS (the force bar), and their sums against the physical
    nonbonded energy."""
    g, gpu, f, e = case
    ea, va = gpu.atom_tallies()
    assert np.sqrt(((ea - g["eatom"]) ** 2).sum() / (g["eatom"] ** 2).sum()) < 1e-9
    assert np.sqrt(((va - g["vatom"]) ** 2).sum() / (g["vatom"] ** 2).sum()) < 1e-9
    assert abs(ea.sum() - 0.5 * (e["e_vdW"] + e["e_ele"])) <= 1e-9 * abs(ea).sum()


def test_gpu_energies_vs_reference(case):
    g, gpu, f, e = case
    ref = dict(zip([str(s) for s in g["energy_names"]], g["energies"]))
    for k in TERMS:
        assert abs(e[k] - ref[k]) <= max(1e-9 * abs(ref[k]), 1e-7), (k, e[k], ref[k])


def test_gpu_forces_vs_reference(case):
    g, gpu, f, e = case
    fr = g["forces"]
    assert np.sqrt(((f - fr) ** 2).sum() / (fr ** 2).sum()) < 1e-9


def test_gpu_lists_vs_reference(case):
    g, gpu, f, e = case
    ti, tj, im, bo = gpu.bond_list()
    assert keyset(ti, tj, im) == keyset(g["bond_ti"], g["bond_tj"], g["bond_img"])
    ref = {k: v for k, v in zip(zip(g["bond_ti"].tolist(), g["bond_tj"].tolist(),
                                    g["bond_img"].tolist()), g["bond_bo"])}
    for k, v in zip(zip(ti.tolist(), tj.tolist(), im.tolist()), bo):
        np.testing.assert_allclose(v, ref[k], rtol=1e-10, atol=1e-13)
    assert keyset(*gpu.hbond_list()) == keyset(g["hb_ti"], g["hb_tj"], g["hb_img"])


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_gpu_qeq_vs_reference(path, ffield):
    g = dict(np.load(path))
    gpu = ReaxGPU(ffield)
    gpu.set_box(g["box"])
    gpu.set_atoms(g["x"], g["types"], g["tags"], None, g["v"])
    q, its, itt = gpu.qeq()
    assert np.abs(q - g["q"]).max() < 1e-5
    assert abs(q.sum()) < 1e-9 * len(q)
    # same CG from the same guesses: iteration counts within one of the
    # reference's (the reduction order of the dot products differs)
    assert abs(its - int(g["qeq_iters"][0])) <= 1 and abs(itt - int(g["qeq_iters"][1])) <= 1


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_gpu_nve_vs_reference(path, ffield):
    g = dict(np.load(path))
    gpu = ReaxGPU(ffield)
    gpu.set_box(g["box"])
    gpu.set_atoms(g["x"], g["types"], g["tags"], None, g["v"])
    e = gpu.run(int(g["nve_steps"]), float(g["nve_dt"]))
    x, v, q, f = gpu.get_atoms()
    box = g["box"]
    dx = x - g["nve_x"]
    dx -= box * np.round(dx / box)
    assert np.abs(dx).max() < 1e-7
    assert np.abs(v - g["nve_v"]).max() < 1e-7
    # along a trajectory the CG starts from extrapolated guesses and stops
    # at the 1e-6 relative residual, where its iterate is up to ~2e-5 e from
    # the converged charges; sums in another order can stop it one iteration
    # earlier or later than the reference, so the bound is the solver's own
    # error (single solves from the same guesses are held to 1e-5 above)
    assert np.abs(q - g["nve_q"]).max() < 5e-5
    ref = dict(zip([str(s) for s in g["energy_names"]], g["nve_energies"]))
    etot = e["eng_vdwl"] + e["eng_coul"]
    etot_r = ref["eng_vdwl"] + ref["eng_coul"]
    assert abs(etot - etot_r) < 1e-6 * abs(etot_r)
