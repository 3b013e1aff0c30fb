"""CPU oracle self-checks: force = -dE/dx by finite differences, momentum
conservation, charge neutrality, list statistics, force-field reading."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import systems

ELEMENTS = ["C", "H", "O", "N"]


@pytest.fixture(scope="module")
def mix(ffield):
    s = systems.mixture(scale=0.0006, seed=3)
    o = Oracle(ffield)
    t = s.types(ELEMENTS)
    o.set_system(s.box, s.x, t, s.tag, None, s.v)
    q, its, itt = o.qeq()
    return s, o, t, q, its, itt


def test_ffield_read(ffield):
    o = Oracle(ffield)
    assert o.type_param(0, "mass") == 12.0
    assert o.type_param(1, "p_hbond") == 1
    assert o.type_param(2, "p_hbond") == 2
    # eta is stored doubled (reaxc_ffield_sunway.cpp:190)
    assert abs(o.type_param(2, "eta") - 2 * 7.1412) < 1e-12


def test_qeq_neutral_and_converged(mix):
    s, o, t, q, its, itt = mix
    assert abs(q.sum()) < 1e-10
    assert 1 < its < 200 and 1 < itt < 200
    assert (q[np.array(s.elem) == "O"] < 0).all()


def test_momentum_conserved(mix):
    s, o, t, q, *_ = mix
    o.set_system(s.box, s.x, t, s.tag, q, s.v)
    f, e = o.compute()
    assert np.abs(f.sum(0)).max() < 1e-9 * np.abs(f).max() * len(f)


def test_forces_are_energy_gradient(mix):
    s, o, t, q, *_ = mix

    def energy(x):
        o.set_system(s.box, x, t, s.tag, q, s.v)
        f, e = o.compute()
        return e["eng_vdwl"] + e["eng_coul"], f

    _, f0 = energy(s.x)
    rng = np.random.default_rng(1)
    h = 1e-5
    for a in rng.choice(s.n, 4, replace=False):
        for d in range(3):
            xp, xm = s.x.copy(), s.x.copy()
            xp[a, d] += h
            xm[a, d] -= h
            fd = -(energy(xp)[0] - energy(xm)[0]) / (2 * h)
            assert abs(fd - f0[a, d]) < 1e-4 * max(1.0, abs(f0[a, d])), (a, d, fd, f0[a, d])


def test_list_statistics(mix):
    s, o, t, q, *_ = mix
    o.set_system(s.box, s.x, t, s.tag, q, s.v)
    o.compute()
    st = o.stats()
    rho = s.n / np.prod(s.box)
    expect = 4.0 / 3.0 * np.pi * 1000.0 * rho
    assert 0.8 * expect < st["n_far_local"] / s.n < 1.2 * expect
    assert st["n_bonds_local"] > s.n
    assert st["n_total"] > st["n_local"]


@pytest.mark.parametrize("swb", [9.0, 10.0, 11.0])
def test_qeq_h_pairs_within_swb(ffield, swb):
    """The QEq H holds every (local atom, partner image) pair within the
    taper radius once, below and above the nonbonded cutoff (above it the
    pairs come from all ghosts, as the fix's own neighbour list reaches the
    pair cutoff plus the skin); counted here by brute force over images."""
    s = systems.water_box(60, seed=2)          # 180 atoms, edge ~12.1 A
    o = Oracle(ffield, qeq_swb=swb)
    o.set_system(s.box, s.x, s.types(ELEMENTS), s.tag, None, s.v)
    o.qeq()
    L = np.asarray(s.box, float)
    x = np.asarray(s.x, float) % L
    count = 0
    r = range(-2, 3)
    for sx in r:
        for sy in r:
            for sz in r:
                d = x[None, :, :] + np.array([sx, sy, sz]) * L - x[:, None, :]
                d2 = (d ** 2).sum(-1)
                ok = d2 <= swb * swb
                if sx == sy == sz == 0:
                    np.fill_diagonal(ok, False)
                count += int(ok.sum())
    assert o.stats()["n_H_entries"] == count
