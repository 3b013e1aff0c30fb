"""Generate golden fixtures from the reference's own CPU code.

Run in a checkout that has the reference sources (the reference is compiled
by oracle/ref/Makefile into oracle/_ref/libreax_ref.so):

    make -C oracle/ref REF=<reference source tree> && python tests/golden/make_golden.py

For each seeded system it stores the inputs (box, positions, types, tags,
charges) and the outputs of the reference's host-side routines run on the
oracle's lists: the 14-term energy vector plus eng_vdwl/eng_coul, the
per-atom forces, the per-atom energy and virial tallies (eatom, vatom of
eflag_atom / vflag_atom), the corrected bond orders of every bond entry (tag_i,
tag_j, image) and the H-bond partner list.  Charges are the reference's
own QEq (FixQEqReaxSunway::pre_force -> init_matvec, CG_v2, calculate_Q,
compiled from fix_qeq_reax_sunway.cpp by oracle/ref/Makefile) from zero
histories, on the H matrix the oracle builds; they are the force step's
input and the QEq's golden output (`q`, `qeq_iters`).  `nve_*` hold the
state after 5 NVE steps of 0.25 fs from the fixture's positions and
velocities, with every step's charges from the reference's QEq (warm
s/t histories).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import ENERGY_NAMES, Oracle, ref_available  # noqa: E402
from sw_reaxff_gb300 import systems  # noqa: E402
from sw_reaxff_gb300.api import DEFAULT_FFIELD  # noqa: E402

CASES = {
    "water600": lambda: systems.water_box(200, seed=1),
    "mixture1k": lambda: systems.mixture(scale=0.001, seed=3),
    "smallbox63": lambda: systems.small_pack(60, 0.8, seed=5),
    "co2pack305": lambda: systems.small_pack(300, 0.6, seed=9),
}
ELEMENTS = ["C", "H", "O", "N"]
NVE_STEPS = 5
NVE_DT = 0.25


def main():
    if not ref_available():
        raise SystemExit("oracle/_ref/libreax_ref.so missing: run make -C oracle/ref first")
    for name, make in CASES.items():
        s = make()
        types = s.types(ELEMENTS)
        o = Oracle(DEFAULT_FFIELD, reference_qeq=True)
        o.set_system(s.box, s.x, types, s.tag, None, s.v)
        q, its, itt = o.qeq()
        o.set_system(s.box, s.x, types, s.tag, q, s.v)
        o.compute()
        ti, tj, im, _ = o.bond_list()
        f, e, bo, hb = o.ref_compute()
        eatom, vatom = o.atom_tallies(reference=True)
        md = Oracle(DEFAULT_FFIELD, reference_qeq=True)
        md.set_system(s.box, s.x, types, s.tag, None, s.v)
        e_md = md.run_nve(NVE_STEPS, NVE_DT)
        x5, v5, q5, f5 = md.state()
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            box=s.box, x=s.x, types=types, tags=s.tag, q=q,
            energies=np.array([e[k] for k in ENERGY_NAMES]), energy_names=np.array(ENERGY_NAMES),
            forces=f, eatom=eatom, vatom=vatom, bond_ti=ti, bond_tj=tj, bond_img=im, bond_bo=bo,
            hb_ti=hb[0], hb_tj=hb[1], hb_img=hb[2], qeq_iters=np.array([its, itt]),
            v=s.v, nve_steps=np.array(NVE_STEPS), nve_dt=np.array(NVE_DT),
            nve_x=x5, nve_v=v5, nve_q=q5, nve_f=f5,
            nve_energies=np.array([e_md[k] for k in ENERGY_NAMES]))
        print(name, s.n, "bonds", len(ti), "hbond partners", len(hb[0]))


if __name__ == "__main__":
    main()
