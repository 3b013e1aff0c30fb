"""rg_single_point: QEq + force step of many independent systems (segments),
replayed as one captured CUDA graph once the same arrays were seen twice --
binning, lists, the QEq's CG iterations (device-side WHILE loops, and in
the mixed form the refinement restarts as nested conditionals) and the
force step, with one host synchronisation.  Replays must give the regular
path's results (within the batch tolerance of test_gpu_batch.py: charges
1e-5 e, forces 1e-5 relative RMS, energies 1e-5 relative), count as
replays, and a replay that meets a list past its capacity must restore the
QEq histories and redo the step on the regular path."""
import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import PREC_MIXED
from sw_reaxff_gb300.systems import System

pytestmark = pytest.mark.gpu
TERMS = ["e_bond", "e_ovun", "e_ang", "e_tor", "e_hb", "e_vdW", "e_ele", "eng_vdwl", "eng_coul"]


def batch():
    rng = np.random.default_rng(12)
    return [systems.small_pack(int(rng.integers(50, 700)), float(rng.uniform(0.4, 1.0)),
                               seed=500 + k) for k in range(24)]


def close(q, f, e, qr, fr, er):
    assert np.abs(q - qr).max() < 1e-5
    assert np.sqrt(((f - fr) ** 2).sum() / (fr ** 2).sum()) < 1e-5
    for k in TERMS:
        assert abs(e[k] - er[k]) <= max(1e-5 * abs(er[k]), 1e-4), (k, e[k], er[k])


@pytest.mark.parametrize("precision", [0, PREC_MIXED], ids=["fp64", "mixed"])
def test_single_point_replays_equal_regular_path(ffield, precision):
    S = batch()
    ref = ReaxGPU(ffield, precision=precision)
    ref.set_systems(S)
    qr, _, _ = ref.qeq()
    fr, er = ref.compute()
    g = ReaxGPU(ffield, precision=precision)
    g.set_systems(S)
    for call in range(5):
        g.set_histories(None, None)          # every call a fresh single point
        q, f, e = g.single_point()
        close(q, f, e, qr, fr, er)
    st = g.stats()
    assert st["step_graph_replays"] >= 3 and st["step_graph_redos"] == 0
    assert st["cg_iters_s"] == ref.stats()["cg_iters_s"] or abs(
        st["cg_iters_s"] - ref.stats()["cg_iters_s"]) <= 1


def test_single_point_overflow_redoes_step(ffield):
    a = systems.water_box(500, density=0.3, seed=61)     # uniform, 0.3 g/cm^3
    b = systems.water_box(500, density=1.0, seed=62)     # a liquid blob ...
    blob = System(box=a.box, x=b.x.copy(), elem=b.elem, tag=b.tag, v=b.v, mol=b.mol)
    g = ReaxGPU(ffield)
    g.set_system(a)
    for _ in range(3):
        g.set_histories(None, None)
        g.single_point()
    assert g.stats()["step_graph_replays"] >= 1
    g.set_positions(blob.x)                               # ... in the same box: lists overflow
    g.set_histories(None, None)
    q, f, e = g.single_point()
    assert g.stats()["step_graph_redos"] == 1
    ref = ReaxGPU(ffield)
    ref.set_system(blob)
    qr, _, _ = ref.qeq()
    fr, er = ref.compute()
    close(q, f, e, qr, fr, er)


def test_repeated_force_steps_agree(ffield):
    """The force step corrects bond orders in place: a second rg_compute on
    the same positions must rebuild the lists and give the same result."""
    s = systems.water_box(120, seed=3)
    g = ReaxGPU(ffield)
    g.set_system(s)
    g.qeq()
    f1, e1 = g.compute()
    f2, e2 = g.compute()
    assert np.sqrt(((f2 - f1) ** 2).sum() / (f1 ** 2).sum()) < 1e-12
    for k in TERMS:
        assert abs(e2[k] - e1[k]) <= 1e-10 * max(abs(e1[k]), 1.0), k


def _handle(ffield, graphs, **kw):
    import os
    old = os.environ.get("RG_NO_GRAPHS")
    os.environ["RG_NO_GRAPHS"] = "0" if graphs else "1"
    try:
        return ReaxGPU(ffield, **kw)
    finally:
        if old is None:
            del os.environ["RG_NO_GRAPHS"]
        else:
            os.environ["RG_NO_GRAPHS"] = old


@pytest.mark.parametrize("precision", [0, PREC_MIXED], ids=["fp64", "mixed"])
def test_md_step_graph_equals_regular_path(ffield, precision):
    """rg_run replays the whole MD step (Verlet half-steps around lists, QEq
    and forces) once it has seen the same arrays twice: 12 steps equal the
    same 12 steps launched phase by phase within 1e-6 A and A/fs, and the
    charges within the CG's stopping error along a trajectory (5e-5 e) --
    the QEq's dot products are summed by atomics in any order, so two runs
    of either path differ by ~1e-7 A and ~1e-5 e after 12 steps (measured)."""
    s = systems.water_box(300, seed=17)
    out = []
    for graphs in (False, True):
        g = _handle(ffield, graphs, precision=precision)
        g.set_system(s)
        g.run(12, 0.25, energies=False)
        out.append(g.get_atoms() + (g.stats(),))
    (x0, v0, q0, _, st0), (x1, v1, q1, _, st1) = out
    assert st0["step_graph_replays"] == 0 and st1["step_graph_replays"] >= 8
    dx = x1 - x0
    dx -= s.box * np.round(dx / s.box)
    assert np.abs(dx).max() < 1e-6 and np.abs(v1 - v0).max() < 1e-6
    assert np.abs(q1 - q0).max() < 5e-5


def test_md_step_overflow_redoes_step(ffield):
    """A replayed MD step whose lists outgrow their capacities restores the
    positions, velocities, forces and QEq histories it started from and redoes
    the step on the regular path."""
    a = systems.water_box(500, density=0.3, seed=61)
    b = systems.water_box(500, density=1.0, seed=62)
    blob = System(box=a.box, x=b.x.copy(), elem=b.elem, tag=b.tag, v=b.v, mol=b.mol)
    ref = ReaxGPU(ffield)                 # the blob's state after a Verlet set-up
    ref.set_system(blob)
    ref.qeq()
    f_b, _ = ref.compute()
    hist = ref.get_histories()
    g = ReaxGPU(ffield)
    g.set_system(a)
    g.run(4, 0.25, energies=False)
    assert g.stats()["step_graph_replays"] >= 1
    g.set_state(blob.x, blob.v, f_b)      # same box, a dense blob: the replay overflows
    g.set_histories(*hist)
    g.run(1, 0.25, energies=False)
    assert g.stats()["step_graph_redos"] == 1
    ref.run(1, 0.25, energies=False)
    x, v, q, f = g.get_atoms()
    xr, vr, qr, fr = ref.get_atoms()
    # (the CG's dot products are FP64 atomics whose order varies from run to
    # run: the charges move by ~1e-9 e and the velocities after the step by
    # ~1e-9)
    assert np.abs(x - xr).max() < 1e-9 and np.abs(v - vr).max() < 1e-7
    assert np.abs(q - qr).max() < 1e-5
