"""rg_qeq_noalloc: the QEq entry point for callers that cannot allocate
device memory when they need charges (code running under a host
application's own device-memory manager, or where an allocation would
synchronize or fail).  It must give the charges of rg_qeq -- within the
1e-5 e bar the QEq parity tests use -- from caller-owned device arrays,
twice in a row (the static scratch array keeps the previous call's
contents), for boxes whose periodic images reach two cells out, for
positions outside the box, and up to its fixed scratch size; and it must
refuse what it cannot do (more atoms than the scratch holds, a box edge
below half the cutoff, a non-finite position, a type outside the force
field) with a message, before any product is formed.
"""
import ctypes as C

import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, systems

pytestmark = pytest.mark.gpu

MAX_ATOMS = 8192   # RG_NOALLOC_MAX_ATOMS in include/reaxgpu.h


def _call(g, n, x, t, box, q):
    its, itt = C.c_int(), C.c_int()
    rc = g.L.rg_qeq_noalloc(g.h, n, x.data_ptr(), t.data_ptr(),
                            box.ctypes.data_as(C.POINTER(C.c_double)), q.data_ptr(),
                            C.byref(its), C.byref(itt), None)
    return rc, its.value, itt.value


def _check_against_rg_qeq(ffield, s, x_in=None):
    """Two calls in a row against rg_qeq's first solve on the same system
    (x_in: positions handed to rg_qeq_noalloc instead of s.x)."""
    torch = pytest.importorskip("torch")
    g = ReaxGPU(ffield)
    g.set_system(s)
    q_ref, its_ref, itt_ref = g.qeq()           # first solve: zero guesses
    types = s.types(g.elements)
    x = torch.tensor(s.x if x_in is None else x_in, dtype=torch.float64, device="cuda")
    t = torch.tensor(types, dtype=torch.int32, device="cuda")
    q = torch.empty(s.n, dtype=torch.float64, device="cuda")
    box = np.ascontiguousarray(s.box, np.float64)
    for call in range(2):
        q.fill_(float("nan"))
        torch.cuda.synchronize()
        rc, its, itt = _call(g, s.n, x, t, box, q)
        assert rc == 0, g.L.rg_last_error(g.h)
        qn = q.cpu().numpy()
        assert np.isfinite(qn).all()
        assert np.abs(qn - q_ref).max() < 1e-5, (call, np.abs(qn - q_ref).max())
        assert abs(qn.sum()) < 1e-9 * max(1, s.n / 1000)
        assert abs(its - its_ref) <= 3 and abs(itt - itt_ref) <= 3


def test_noalloc_qeq_matches_rg_qeq(ffield):
    _check_against_rg_qeq(ffield, systems.water_box(200, seed=1))   # 600 atoms, one image


def test_noalloc_small_box_two_images(ffield):
    s = systems.water_box(11, seed=4)           # 33 atoms, edge 6.9 A: images to +-2
    assert s.box.max() < 10.0 / 1.4
    _check_against_rg_qeq(ffield, s)


def test_noalloc_unwrapped_positions(ffield):
    s = systems.water_box(60, seed=6)           # 180 atoms
    rng = np.random.default_rng(6)
    shift = rng.integers(-3, 4, size=s.x.shape) * s.box
    _check_against_rg_qeq(ffield, s, s.x + shift)


def test_noalloc_near_scratch_limit(ffield):
    s = systems.water_box(2730, seed=8)         # 8190 atoms of the 8192 the scratch holds
    assert MAX_ATOMS - 3 < s.n <= MAX_ATOMS
    _check_against_rg_qeq(ffield, s)


def test_noalloc_rejects_oversize(ffield):
    torch = pytest.importorskip("torch")
    g = ReaxGPU(ffield)
    x = torch.zeros(3, dtype=torch.float64, device="cuda")
    t = torch.zeros(1, dtype=torch.int32, device="cuda")
    q = torch.zeros(1, dtype=torch.float64, device="cuda")
    box = np.array([20.0, 20.0, 20.0])
    rc, _, _ = _call(g, MAX_ATOMS + 1, x, t, box, q)
    assert rc == -1
    assert b"scratch" in g.L.rg_last_error(g.h)


def test_noalloc_rejects_bad_inputs(ffield):
    torch = pytest.importorskip("torch")
    g = ReaxGPU(ffield)
    n = 4
    x = torch.tensor(np.arange(3 * n, dtype=np.float64), device="cuda")
    t = torch.zeros(n, dtype=torch.int32, device="cuda")
    q = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc, _, _ = _call(g, n, x, t, np.array([20.0, 4.0, 20.0]), q)   # edge below 5 A
    assert rc == -1 and b"half the QEq cutoff" in g.L.rg_last_error(g.h)
    rc, _, _ = _call(g, n, x, t, np.array([20.0, np.inf, 20.0]), q)
    assert rc == -1 and b"finite" in g.L.rg_last_error(g.h)
    box = np.array([20.0, 20.0, 20.0])
    xb = x.clone()
    xb[4] = float("nan")
    rc, _, _ = _call(g, n, xb, t, box, q)
    assert rc == -1 and b"not finite" in g.L.rg_last_error(g.h)
    tb = t.clone()
    tb[2] = len(g.elements)
    rc, _, _ = _call(g, n, x, tb, box, q)
    assert rc == -1 and b"type" in g.L.rg_last_error(g.h)
    # the scratch keeps no state that a rejected call spoils
    rc, _, _ = _call(g, n, x, t, box, q)
    assert rc == 0, g.L.rg_last_error(g.h)
