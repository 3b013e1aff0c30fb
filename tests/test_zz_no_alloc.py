"""rg_qeq_noalloc: the QEq entry point for callers that cannot allocate
device memory when they need charges (code running under a host
application's own device-memory manager, or where an allocation would
synchronize or fail).  It must give the charges of rg_qeq -- within the
1e-5 e bar the QEq parity tests use -- from caller-owned device arrays,
twice in a row (the static scratch array keeps the previous call's
contents), and refuse systems beyond its fixed scratch size.
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


def test_noalloc_qeq_matches_rg_qeq(ffield):
    torch = pytest.importorskip("torch")
    s = systems.water_box(200, seed=1)          # 600 atoms, box < 2 x 10 A
    g = ReaxGPU(ffield)
    g.set_system(s)
    q_ref, its_ref, itt_ref = g.qeq()           # first solve: zero guesses
    types = s.types(g.elements)
    x = torch.tensor(s.x, dtype=torch.float64, device="cuda")
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
        assert abs(qn.sum()) < 1e-9
        assert abs(its - its_ref) <= 3 and abs(itt - itt_ref) <= 3


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
