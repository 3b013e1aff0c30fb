"""Host-side logic of the request loop (no GPU): the request stream has the
stated shape (Poisson arrivals, log-uniform sizes within bounds, the MD
fraction and step range) and is reproducible from its seed."""
import math

import numpy as np

from sw_reaxff_gb300 import serve


def test_stream_specs_shape_and_seed():
    a = serve.stream_specs(2000, rate=200.0, seed=3)
    b = serve.stream_specs(2000, rate=200.0, seed=3)
    assert a == b
    arrivals = np.array([s[1] for s in a])
    sizes = np.array([s[2] for s in a])
    dens = np.array([s[3] for s in a])
    kinds = [s[5] for s in a]
    steps = np.array([s[6] for s in a if s[5] == "md"])
    assert np.all(np.diff(arrivals) > 0)
    gaps = np.diff(np.concatenate([[0.0], arrivals]))
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0          # Poisson mean gap
    assert sizes.min() >= 100 and sizes.max() <= 20000
    logs = np.log(sizes)
    assert abs(logs.mean() - 0.5 * (math.log(100) + math.log(20000))) < 0.15
    assert dens.min() >= 0.3 and dens.max() <= 1.0
    frac = kinds.count("md") / len(kinds)
    assert abs(frac - 0.3) < 0.04
    assert steps.min() >= 10 and steps.max() <= 500


def test_make_request_builds_the_system():
    spec = serve.stream_specs(1, rate=10.0, seed=1, max_atoms=300)[0]
    r = serve.make_request(spec)
    assert r.rid == spec[0] and r.kind == spec[5]
    assert abs(r.system.n - spec[2]) <= 8          # whole molecules
    assert np.all(r.system.x >= 0) and np.all(r.system.x < r.system.box)
