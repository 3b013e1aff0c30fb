"""The CUDA force step against the golden fixtures of the reference's own
code (same positions and charges): bond and H-bond lists as sets, corrected
bond orders within 1e-10, per-term energies within 1e-9 relative, forces
within 1e-9 relative RMS."""
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
    f, e = gpu.compute()
    return g, gpu, f, e


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
