"""The request loop (sw_reaxff_gb300/serve.py): continuous batching of single
points and short NVE runs.  Every request completes; each result equals the
same request run alone in the same form within the tolerance stated in
test_gpu_batch.py (the batch only reorders FP64 reductions); MD state is
carried across cohort rebuilds; admission respects the memory budget."""
import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, serve
from sw_reaxff_gb300.api import PREC_MIXED

pytestmark = pytest.mark.gpu

TOL_Q, TOL_F, TOL_X, TOL_V = 1e-5, 1e-5, 1e-5, 1e-5


def stream():
    # small sizes and step counts keep the alone-runs quick; arrivals packed
    # so that requests arrive while others run
    return serve.request_stream(14, rate=400.0, seed=5, min_atoms=60, max_atoms=1500,
                                md_fraction=0.4, md_steps=(3, 25))


def alone(ffield, r, precision):
    g = ReaxGPU(ffield, precision=precision)
    g.set_system(r.system)
    if r.kind == "sp":
        q, _, _ = g.qeq()
        f, e = g.compute()
        return dict(q=q, f=f, e=e)
    g.run(r.nsteps, 0.25, energies=False)
    x, v, q, f = g.get_atoms()
    return dict(x=x, v=v, q=q, f=f)


@pytest.mark.parametrize("precision", [0, PREC_MIXED])
def test_serve_results_equal_alone(ffield, precision):
    reqs = stream()
    srv = serve.ReaxServer(ffield, precision=precision, md_chunk=4)
    st = srv.serve(reqs, realtime=True)
    srv.close()
    assert st.completed == len(reqs)
    assert all(np.isfinite(r.latency) and r.latency >= 0 for r in reqs)
    assert st.rebuilds >= 1
    for r in reqs:
        a = alone(ffield, r, precision)
        if r.kind == "sp":
            assert np.abs(r.q - a["q"]).max() < TOL_Q, r.rid
            rel = np.sqrt(((r.f - a["f"]) ** 2).sum() / (a["f"] ** 2).sum())
            assert rel < TOL_F, (r.rid, rel)
        else:
            L = r.system.box
            dx = r.x - a["x"]
            dx -= L * np.round(dx / L)
            assert np.abs(dx).max() < TOL_X, r.rid
            assert np.abs(r.v - a["v"]).max() < TOL_V, r.rid


def test_serve_admission_budget(ffield):
    reqs = stream()
    big = max(r.system.n for r in reqs)
    # room for about two of the largest requests at a time
    budget = 2 * big * serve.BYTES_PER_ATOM[PREC_MIXED]
    srv = serve.ReaxServer(ffield, precision=PREC_MIXED, hbm_budget=budget, md_chunk=4)
    st = srv.serve(reqs, realtime=False)
    srv.close()
    assert st.completed == len(reqs)
    assert st.max_atoms_on_device <= 2 * big
    s = st.summary()
    assert s["p99_ms"] >= s["p50_ms"] > 0
