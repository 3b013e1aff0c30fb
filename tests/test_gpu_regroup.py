"""rg_regroup_segments / rg_get_segment_atoms: the device-side cohort edits
of continuous batching.  A regroup copies every carried system's state
exactly (positions, velocities, charges, forces and QEq histories: bit for
bit), and MD trajectories continued across regroups -- some systems
leaving, systems of another handle joining -- equal the same trajectories
run alone, within the batch tolerance of test_gpu_batch.py (the batch only
reorders FP64 reductions)."""
import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, systems

pytestmark = pytest.mark.gpu
DT = 0.25


def packs():
    return [systems.small_pack(n, d, seed=s) for n, d, s in
            ((120, 0.8, 41), (300, 0.6, 42), (80, 0.9, 43), (200, 0.7, 44))]


def test_regroup_copies_state_exactly(ffield):
    S = packs()
    a = ReaxGPU(ffield)
    a.set_systems(S[:3])
    a.run(3, DT, energies=False)
    b = ReaxGPU(ffield)
    b.set_systems(S[3:])
    b.qeq()
    b.compute()
    before = {("a", k): a.segment_atoms(k) for k in range(3)}
    before[("b", 0)] = b.segment_atoms(0)
    ha = a.get_histories()
    off_a = np.concatenate([[0], np.cumsum([s.n for s in S[:3]])])
    hb = b.get_histories()
    off = a.regroup([2, 0], b, [0])
    assert list(off) == [0, S[2].n, S[2].n + S[0].n]
    after = [a.segment_atoms(k) for k in range(3)]
    for new, old in zip(after, [before[("a", 2)], before[("a", 0)], before[("b", 0)]]):
        for x, y in zip(new, old):
            assert np.array_equal(x, y)
    s_h, t_h = a.get_histories()
    want_s = np.concatenate([ha[0][:, off_a[2]:off_a[3]], ha[0][:, off_a[0]:off_a[1]], hb[0]], axis=1)
    want_t = np.concatenate([ha[1][:, off_a[2]:off_a[3]], ha[1][:, off_a[0]:off_a[1]], hb[1]], axis=1)
    assert np.array_equal(s_h, want_s) and np.array_equal(t_h, want_t)


def alone(ffield, s, nsteps):
    g = ReaxGPU(ffield)
    g.set_system(s)
    g.run(nsteps, DT, energies=False)
    x, v, q, f = g.get_atoms()
    return x, v, q


def test_trajectories_continue_across_regroups(ffield):
    S = packs()
    cohort = ReaxGPU(ffield)
    cohort.set_systems(S[:3])
    cohort.run(4, DT, energies=False)           # systems 0, 1, 2: 4 steps
    ev = ReaxGPU(ffield)
    ev.set_systems([S[3]])
    ev.qeq()
    ev.compute()                                 # system 3: evaluated, 0 steps
    cohort.regroup([0, 2], ev, [0])              # system 1 leaves, 3 joins
    cohort.run(6, DT, energies=False)
    done = {0: 10, 2: 10, 3: 6}
    for seg, (k, steps) in enumerate(done.items()):
        x, v, q, _ = cohort.segment_atoms(seg)
        xa, va, qa = alone(ffield, S[k], steps)
        L = S[k].box
        dx = x - xa
        dx -= L * np.round(dx / L)
        assert np.abs(dx).max() < 1e-5, (k, np.abs(dx).max())
        assert np.abs(v - va).max() < 1e-5, k
        assert np.abs(q - qa).max() < 5e-5, k


def test_regroup_rejects_bad_indices(ffield):
    S = packs()
    a = ReaxGPU(ffield)
    a.set_systems(S[:2])
    with pytest.raises(Exception):
        a.regroup([5])
    b = ReaxGPU(ffield)
    with pytest.raises(Exception):
        a.regroup([0], b, [0])                   # b holds no atoms
