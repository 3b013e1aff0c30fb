"""Generate the 6,000-atom water trajectory fixture (traj/water6k_nve100.npz).

The workload: 2,000 H2O at 1.0 g/cm^3 (sw_reaxff_gb300.systems.water_box,
seed 2024), 300 K velocities, the CHON force field with the reference's
default cutoffs (10 A nonbonded, 5 A bond, 7.5 A H-bond, bond-order cutoff
1e-4), QEq tolerance 1e-6, 100 velocity-Verlet steps of 0.25 fs.  The
trajectory is the oracle's, with every step's charges from the reference's
own QEq driver (oracle/ref: FixQEqReaxSunway::pre_force compiled from the
reference sources), so the run needs oracle/_ref/libreax_ref.so:

    make -C oracle/ref REF=<reference source tree> && python tests/golden/make_trajectory.py

Stored: the initial state (box, x, v, types, tags; stored rather than
regenerated so that a test does not depend on the generator's floating
point on another machine), the state after 100 steps (x, v, q, f) and the
energy vector of the last step.  About two and a half minutes on one core.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import ENERGY_NAMES, Oracle, ref_available  # noqa: E402
from sw_reaxff_gb300 import systems  # noqa: E402
from sw_reaxff_gb300.api import DEFAULT_FFIELD  # noqa: E402

ELEMENTS = ["C", "H", "O", "N"]
STEPS = 100
DT = 0.25
OUT = os.path.join(HERE, "traj", "water6k_nve100.npz")


def main():
    if not ref_available():
        raise SystemExit("oracle/_ref/libreax_ref.so missing: run make -C oracle/ref first")
    s = systems.water_box(2000, seed=2024)
    types = s.types(ELEMENTS)
    o = Oracle(DEFAULT_FFIELD, reference_qeq=True)
    o.set_system(s.box, s.x, types, s.tag, None, s.v)
    t0 = time.time()
    e = o.run_nve(STEPS, DT)
    x, v, q, f = o.state()
    np.savez_compressed(OUT, box=s.box, x0=s.x, v0=s.v, types=types, tags=s.tag,
                        steps=np.array(STEPS), dt=np.array(DT), x=x, v=v, q=q, f=f,
                        energies=np.array([e[k] for k in ENERGY_NAMES]),
                        energy_names=np.array(ENERGY_NAMES))
    print(f"{s.n} atoms, {STEPS} steps in {time.time() - t0:.0f} s -> {OUT}")


if __name__ == "__main__":
    main()
