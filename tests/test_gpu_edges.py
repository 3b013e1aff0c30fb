"""Edge cases of the C ABI on the GPU: calls in the wrong order and invalid
inputs return error codes with messages (the reference aborts through
error->all / MPI_Abort); tiny, empty-bond and single-species systems run
and agree with the oracle; boxes at the smallest supported width work and
narrower ones are refused."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import ReaxError

pytestmark = pytest.mark.gpu

ELS = ["C", "H", "O", "N"]


def test_call_order_and_arguments(ffield):
    g = ReaxGPU(ffield)
    with pytest.raises(ReaxError, match="no atoms"):
        g.qeq()
    with pytest.raises(ReaxError):
        g.bond_table()                      # no force step yet
    g.set_box([20.0, 20.0, 20.0])
    with pytest.raises(ReaxError):
        g.set_atoms(np.zeros((2, 3)), np.array([0, 9], np.int32))   # type out of range
    with pytest.raises(ReaxError, match="box"):
        g.set_box([20.0, -1.0, 20.0])
    with pytest.raises(ReaxError, match="non-finite"):
        g.set_atoms(np.array([[1.0, np.nan, 1.0]]), np.array([0], np.int32))
    with pytest.raises(Exception):
        g.set_systems([])                   # no segments
    with pytest.raises(Exception):
        ReaxGPU(ffield, cell_div=5)          # invalid configuration
    with pytest.raises(Exception):
        ReaxGPU("/nonexistent/ffield")


def test_box_narrower_than_half_cutoff_is_refused(ffield):
    g = ReaxGPU(ffield)
    g.set_box([4.0, 20.0, 20.0])             # 4 A < 10 A / 2
    g.set_atoms(np.array([[1.0, 1.0, 1.0], [2.0, 2.0, 2.0]]), np.array([1, 1], np.int32))
    with pytest.raises(ReaxError, match="half the pair cutoff"):
        g.qeq()


def check_vs_oracle(ffield, box, x, types, tol_f=1e-9):
    g = ReaxGPU(ffield)
    g.set_box(box)
    g.set_atoms(x, types)
    o = Oracle(ffield)
    o.set_system(np.asarray(box, float), x, types)
    qo, _, _ = o.qeq()
    fo, eo = o.compute()
    qg, _, _ = g.qeq()
    assert np.abs(qg - qo).max() < 1e-5
    g.set_atoms(x, types, None, qo)
    fg, eg = g.compute()
    scale = max(np.sqrt((fo ** 2).sum()), 1e-12)
    assert np.sqrt(((fg - fo) ** 2).sum()) <= tol_f * scale + 1e-9
    for k in ("eng_vdwl", "eng_coul", "e_bond", "e_vdW", "e_ele"):
        assert abs(eg[k] - eo[k]) <= 1e-9 * max(1.0, abs(eo[k])), k
    return g


def test_two_atoms_no_bonds(ffield):
    # two O atoms 4 A apart: nonbonded and QEq only, no bond, angle or torsion
    x = np.array([[5.0, 5.0, 5.0], [9.0, 5.0, 5.0]])
    g = check_vs_oracle(ffield, [12.0, 12.0, 12.0], x, np.array([2, 2], np.int32))
    assert g.stats()["n_bonds"] == 0


def test_single_atom_self_images(ffield):
    # one atom in a 6 A box: every partner is a periodic image of itself
    x = np.array([[1.0, 2.0, 3.0]])
    check_vs_oracle(ffield, [6.0, 6.0, 6.0], x, np.array([0], np.int32))


def test_pure_hydrogen_gas(ffield):
    # random H atoms at least 0.8 A apart (periodic): H2 molecules form
    rng = np.random.default_rng(3)
    L = 14.0
    pts = []
    while len(pts) < 60:
        p = rng.uniform(0, L, 3)
        dd = [np.linalg.norm((p - q + L / 2) % L - L / 2) for q in pts]
        if not dd or min(dd) > 0.8:
            pts.append(p)
    check_vs_oracle(ffield, [L, L, L], np.array(pts), np.ones(60, np.int32))


def test_positions_outside_box_are_wrapped(ffield):
    s = systems.water_box(60, seed=2)
    shift = np.array([3.0, -2.0, 1.0])[None, :] * s.box[None, :]
    g1 = ReaxGPU(ffield)
    g1.set_box(s.box)
    g1.set_atoms(s.x, s.types(g1.elements))
    q1, _, _ = g1.qeq()
    f1, e1 = g1.compute()
    g2 = ReaxGPU(ffield)
    g2.set_box(s.box)
    g2.set_atoms(s.x + shift, s.types(g2.elements))
    q2, _, _ = g2.qeq()
    f2, e2 = g2.compute()
    # the wrapped coordinates differ from s.x by rounding only
    assert np.abs(q2 - q1).max() < 1e-5
    assert np.sqrt(((f2 - f1) ** 2).sum() / (f1 ** 2).sum()) < 1e-5
