"""Virial (row a11: the pressure part of the force copy-out,
pair_reaxc_sunway.cpp:674-763).  With fixed charges, the diagonal of
W = sum r (x) f is minus the derivative of the potential energy under a
uniform stretch of one box edge (positions scaled with it); checked by
central differences in the FP64 form, per segment in a batch, and against
the FP64 form for the mixed form."""
import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import PREC_MIXED

pytestmark = pytest.mark.gpu

CASES = {"water600": lambda: systems.water_box(200, seed=1),
         "mixture1k": lambda: systems.mixture(scale=0.001, seed=3),
         "pack300": lambda: systems.small_pack(300, 0.9, seed=7)}


def charges(ffield, s):
    g = ReaxGPU(ffield)
    g.set_system(s)
    return g.qeq()[0]


def energy_virial(ffield, s, q, stretch=(1.0, 1.0, 1.0), **kw):
    g = ReaxGPU(ffield, **kw)
    st = np.asarray(stretch)
    g.set_box(s.box * st)
    g.set_atoms(s.x * st, s.types(g.elements), s.tag, q, s.v)
    f, e = g.compute(eflag=1, vflag=1)
    return e["eng_vdwl"] + e["eng_coul"], g.virial()[0], f


@pytest.mark.parametrize("case", list(CASES))
def test_virial_diagonal_is_strain_derivative(ffield, case):
    s = CASES[case]()
    q = charges(ffield, s)
    _, W, _ = energy_virial(ffield, s, q)
    eps = 1e-6
    for a in range(3):
        up = np.ones(3); up[a] += eps
        dn = np.ones(3); dn[a] -= eps
        dE = (energy_virial(ffield, s, q, up)[0] - energy_virial(ffield, s, q, dn)[0]) / (2 * eps)
        assert abs(W[a] + dE) <= 1e-5 * max(abs(dE), 1.0), (a, W[a], -dE)


def test_virial_per_segment_equals_alone(ffield):
    S = [CASES[k]() for k in CASES]
    qs = [charges(ffield, s) for s in S]
    g = ReaxGPU(ffield)
    counts = [s.n for s in S]
    g.set_systems(S)
    g.set_atoms(np.concatenate([s.x for s in S]), np.concatenate([s.types(g.elements) for s in S]),
                np.concatenate([s.tag for s in S]), np.concatenate(qs),
                np.concatenate([s.v for s in S]))
    g.compute(eflag=1, vflag=1)
    Wb = g.virial()
    assert Wb.shape == (len(S), 6)
    for k, s in enumerate(S):
        _, Wa, _ = energy_virial(ffield, s, qs[k])
        assert np.abs(Wb[k] - Wa).max() <= 1e-8 * np.abs(Wa).max(), k
    assert counts


def test_mixed_virial_close_to_fp64(ffield):
    s = CASES["mixture1k"]()
    q = charges(ffield, s)
    _, W64, _ = energy_virial(ffield, s, q)
    _, W32, _ = energy_virial(ffield, s, q, precision=PREC_MIXED)
    assert np.abs(W32 - W64).max() <= 1e-4 * np.abs(W64).max()
