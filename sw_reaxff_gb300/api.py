"""ctypes binding of libreaxgpu.so (the C ABI in include/reaxgpu.h).

The library is the product: every call here goes to the CUDA kernels.  If
the shared library cannot be loaded the import of this module's classes
fails loudly; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libreaxgpu.so")
DEFAULT_FFIELD = os.path.join(HERE, "data", "ffield.reax")

ENERGY_NAMES = ["e_bond", "e_ovun", "e_lp", "e_3", "e_ang", "e_pen", "e_coa",
                "e_hb", "e_tor", "e_con", "e_vdW", "e_ele", "e_12", "e_pol",
                "eng_vdwl", "eng_coul", "e_pol_phys"]
NENERGY = len(ENERGY_NAMES)

PREC_FP64, PREC_MIXED = 0, 1

EXPORTED = ["rg_default_params", "rg_create", "rg_destroy", "rg_last_error",
            "rg_num_types", "rg_element_name", "rg_extract", "rg_set_box", "rg_set_tilt",
            "rg_set_atoms", "rg_set_atoms_device", "rg_set_positions", "rg_qeq",
            "rg_compute", "rg_nve_initial", "rg_nve_final", "rg_run",
            "rg_get_atoms", "rg_device_arrays", "rg_get_stats", "rg_synchronize",
            "rg_dump_pairs", "rg_dump_bonds", "rg_dump_hbonds", "rg_set_state",
            "rg_stream", "rg_profile_enable", "rg_profile_get", "rg_profile_phases",
            "rg_measure_fp64_peak",
            "rg_qeq_noalloc", "rg_set_masses", "rg_ffield_info", "rg_set_segments",
            "rg_num_segments", "rg_get_energies", "rg_get_segment_iters",
            "rg_get_histories", "rg_set_histories", "rg_table_info", "rg_table_check",
            "rg_get_virial", "rg_bond_table", "rg_get_atom_tallies",
            "rg_regroup_segments", "rg_get_segment_atoms", "rg_single_point"]


class Params(C.Structure):
    _fields_ = [("bond_cut", C.c_double), ("hbond_cut", C.c_double),
                ("thb_cut", C.c_double), ("thb_cutsq", C.c_double),
                ("enobondsflag", C.c_int), ("lgflag", C.c_int),
                ("qeq_swa", C.c_double), ("qeq_swb", C.c_double),
                ("qeq_tol", C.c_double), ("qeq_imax", C.c_int),
                ("precision", C.c_int), ("device", C.c_int), ("tabulate", C.c_int),
                ("tabulate_check", C.c_int), ("autotune", C.c_int), ("cell_div", C.c_int),
                ("spmv_rows", C.c_int), ("pair_kernel", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("n_atoms", C.c_longlong), ("n_pairs", C.c_longlong),
                ("n_bonds", C.c_longlong), ("n_hbond_pairs", C.c_longlong),
                ("n_H_entries", C.c_longlong), ("cg_iters_s", C.c_int),
                ("cg_iters_t", C.c_int), ("max_nbrs", C.c_int),
                ("max_bonds", C.c_int), ("max_hbonds", C.c_int),
                ("regrows", C.c_int), ("kernel_launches", C.c_longlong),
                ("qeq_restarts", C.c_int), ("fp64_angles", C.c_int),
                ("fp64_torsions", C.c_int), ("cell_div", C.c_int), ("spmv_rows", C.c_int),
                ("cg_system_iters", C.c_longlong), ("cg_spmv_rows_passes", C.c_longlong),
                ("step_graph_replays", C.c_longlong), ("step_graph_redos", C.c_longlong),
                ("pair_kernel", C.c_int)]


class ReaxError(RuntimeError):
    pass


_lib = None


def load_library(path: str = LIBPATH):
    """Load libreaxgpu.so and declare its C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ReaxError(f"{path} is missing: build it with "
                        "`python sw_reaxff_gb300/build.py` (or __graft_entry__.build())")
    L = C.CDLL(path)
    P = C.POINTER
    dp, ip = P(C.c_double), P(C.c_int)
    L.rg_default_params.argtypes = [P(Params)]
    L.rg_create.argtypes = [C.c_char_p, P(Params), P(C.c_void_p)]
    L.rg_destroy.argtypes = [C.c_void_p]
    L.rg_last_error.restype = C.c_char_p
    L.rg_last_error.argtypes = [C.c_void_p]
    L.rg_num_types.argtypes = [C.c_void_p]
    L.rg_element_name.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
    L.rg_extract.argtypes = [C.c_void_p, C.c_char_p, dp]
    L.rg_set_box.argtypes = [C.c_void_p, dp]
    L.rg_set_tilt.argtypes = [C.c_void_p, dp]
    L.rg_set_masses.argtypes = [C.c_void_p, dp]
    L.rg_set_segments.argtypes = [C.c_void_p, C.c_int, ip, dp]
    L.rg_num_segments.argtypes = [C.c_void_p]
    L.rg_get_energies.argtypes = [C.c_void_p, dp]
    L.rg_get_segment_iters.argtypes = [C.c_void_p, ip]
    L.rg_get_histories.argtypes = [C.c_void_p, dp, dp]
    L.rg_table_info.argtypes = [C.c_void_p, ip, dp]
    L.rg_get_virial.argtypes = [C.c_void_p, dp]
    L.rg_get_atom_tallies.argtypes = [C.c_void_p, dp, dp]
    L.rg_regroup_segments.argtypes = [C.c_void_p, C.c_int, ip, C.c_void_p, C.c_int, ip]
    L.rg_get_segment_atoms.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
    L.rg_single_point.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp, dp]
    L.rg_bond_table.argtypes = [C.c_void_p, C.c_double, C.c_int, ip, ip, dp, dp, dp]
    L.rg_table_check.argtypes = [C.c_char_p, P(Params), dp]
    L.rg_set_histories.argtypes = [C.c_void_p, dp, dp]
    L.rg_ffield_info.argtypes = [C.c_char_p, ip, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    L.rg_set_atoms.argtypes = [C.c_void_p, C.c_int, dp, ip, ip, dp, dp]
    L.rg_set_atoms_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    L.rg_set_positions.argtypes = [C.c_void_p, dp]
    L.rg_qeq.argtypes = [C.c_void_p, dp, ip, ip]
    L.rg_compute.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp]
    L.rg_nve_initial.argtypes = [C.c_void_p, C.c_double]
    L.rg_nve_final.argtypes = [C.c_void_p, C.c_double]
    L.rg_run.argtypes = [C.c_void_p, C.c_int, C.c_double, dp]
    L.rg_get_atoms.argtypes = [C.c_void_p, dp, dp, dp, dp]
    L.rg_device_arrays.argtypes = [C.c_void_p] + [P(C.c_void_p)] * 4
    L.rg_get_stats.argtypes = [C.c_void_p, P(Stats)]
    L.rg_synchronize.argtypes = [C.c_void_p]
    for f in ("rg_dump_pairs", "rg_dump_hbonds"):
        getattr(L, f).restype = C.c_longlong
        getattr(L, f).argtypes = [C.c_void_p, ip, ip, ip]
    L.rg_dump_bonds.restype = C.c_longlong
    L.rg_dump_bonds.argtypes = [C.c_void_p, ip, ip, ip, dp]
    L.rg_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.rg_stream.restype = C.c_void_p
    L.rg_stream.argtypes = [C.c_void_p]
    L.rg_profile_enable.argtypes = [C.c_void_p, C.c_int]
    L.rg_profile_phases.argtypes = [C.c_void_p, C.c_uint]
    L.rg_profile_get.argtypes = [C.c_void_p, C.c_int, C.c_char_p, dp, P(C.c_longlong)]
    L.rg_measure_fp64_peak.argtypes = [C.c_int, dp]
    L.rg_qeq_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, dp,
                                 C.c_void_p, ip, ip, C.c_void_p]
    _lib = L
    return L


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def measure_fp64_peak(device: int = 0) -> float:
    """FP64 FMA throughput of the device in TFLOP/s."""
    L = load_library()
    t = C.c_double()
    if L.rg_measure_fp64_peak(device, C.byref(t)) != 0:
        raise ReaxError("rg_measure_fp64_peak failed")
    return t.value


def ffield_elements(path: str = None) -> list:
    """Element names of a force-field file (host only, no device)."""
    L = load_library()
    n = C.c_int()
    msg = C.create_string_buffer(256)
    if L.rg_ffield_info((path or DEFAULT_FFIELD).encode(), C.byref(n), None, 0, msg, 256) != 0:
        raise ReaxError(msg.value.decode())
    buf = C.create_string_buffer(16 * n.value)
    L.rg_ffield_info((path or DEFAULT_FFIELD).encode(), C.byref(n), buf, 16, None, 0)
    return [buf.raw[16 * k:16 * (k + 1)].split(b"\0")[0].decode() for k in range(n.value)]


def default_params(**kw) -> Params:
    L = load_library()
    p = Params()
    L.rg_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class ReaxGPU:
    """One periodic system on one GPU, driven through the C ABI."""

    def __init__(self, ffield: str = DEFAULT_FFIELD, **params):
        self.L = load_library()
        self.params = default_params(**params)
        h = C.c_void_p()
        rc = self.L.rg_create(ffield.encode(), C.byref(self.params), C.byref(h))
        if rc != 0:
            raise ReaxError(f"rg_create failed ({rc}) for {ffield}")
        self.h = h
        self.n = 0
        self.elements = []
        buf = C.create_string_buffer(16)
        for t in range(self.L.rg_num_types(h)):
            self.L.rg_element_name(h, t, buf, 16)
            self.elements.append(buf.value.decode())

    def _chk(self, rc, what):
        if rc != 0:
            msg = self.L.rg_last_error(self.h)
            raise ReaxError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self.L.rg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def extract(self, name: str) -> np.ndarray:
        out = np.zeros(len(self.elements))
        self._chk(self.L.rg_extract(self.h, name.encode(), _dp(out)), "rg_extract")
        return out

    def set_masses(self, masses):
        """Integrator masses per ffield type (default: the force field's)."""
        m = np.ascontiguousarray(masses, np.float64)
        if m.shape != (len(self.elements),):
            raise ValueError("one mass per force-field type")
        self._chk(self.L.rg_set_masses(self.h, _dp(m)), "rg_set_masses")

    def set_box(self, box):
        box = np.ascontiguousarray(box, np.float64)
        self._chk(self.L.rg_set_box(self.h, _dp(box)), "rg_set_box")
        self._seg_counts = None
        self.nseg = 1

    def set_atoms(self, x, types, tags=None, q=None, v=None):
        x = np.ascontiguousarray(x, np.float64)
        n = x.shape[0]
        types = np.ascontiguousarray(types, np.int32)
        tags = None if tags is None else np.ascontiguousarray(tags, np.int32)
        q = None if q is None else np.ascontiguousarray(q, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        self._chk(self.L.rg_set_atoms(self.h, n, _dp(x), _ip(types), _ip(tags), _dp(q), _dp(v)),
                  "rg_set_atoms")
        self.n = n
        if sum(getattr(self, "_seg_counts", None) or []) != n:
            self._seg_counts = [n]

    def set_tilt(self, tilt):
        """Tilts (xy, xz, yz) of a triclinic box, one row per segment."""
        tl = np.ascontiguousarray(tilt, np.float64).reshape(-1)
        self._chk(self.L.rg_set_tilt(self.h, _dp(tl)), "rg_set_tilt")

    def set_system(self, system):
        """Load a sw_reaxff_gb300.systems.System."""
        self.set_box(system.box)
        if system.triclinic:
            self.set_tilt(system.tilt)
        self.set_atoms(system.x, system.types(self.elements), system.tag, None, system.v)

    def set_systems(self, systems_list):
        """Load several independent systems as segments of one handle
        (batched evaluation): every call then works on all of them.
        Returns the atom offset of each system in the concatenated arrays."""
        counts = np.array([s.n for s in systems_list], np.int32)
        boxes = np.ascontiguousarray(np.stack([s.box for s in systems_list]), np.float64)
        self._chk(self.L.rg_set_segments(self.h, len(systems_list), _ip(counts), _dp(boxes)),
                  "rg_set_segments")
        if any(s.triclinic for s in systems_list):
            self.set_tilt(np.stack([np.zeros(3) if s.tilt is None else np.asarray(s.tilt, float)
                                    for s in systems_list]))
        x = np.concatenate([s.x for s in systems_list])
        types = np.concatenate([s.types(self.elements) for s in systems_list])
        tags = np.concatenate([s.tag for s in systems_list])
        v = np.concatenate([s.v for s in systems_list])
        self.set_atoms(x, types, tags, None, v)
        self.nseg = len(systems_list)
        self._seg_counts = [int(c) for c in counts]
        return np.concatenate([[0], np.cumsum(counts)[:-1]])

    def energies(self):
        """Per-segment energy vectors of the last force step (dicts)."""
        ns = self.L.rg_num_segments(self.h)
        e = np.zeros((ns, NENERGY))
        self._chk(self.L.rg_get_energies(self.h, _dp(e)), "rg_get_energies")
        return [dict(zip(ENERGY_NAMES, row)) for row in e]

    def segment_iters(self):
        """(s, t) CG iterations of the last QEq per segment."""
        ns = self.L.rg_num_segments(self.h)
        it = np.zeros(2 * ns, np.int32)
        self._chk(self.L.rg_get_segment_iters(self.h, _ip(it)), "rg_get_segment_iters")
        return it.reshape(ns, 2)

    def get_histories(self):
        """QEq histories, two (5, n) arrays (latest solve first)."""
        s = np.zeros((5, self.n))
        t = np.zeros((5, self.n))
        self._chk(self.L.rg_get_histories(self.h, _dp(s), _dp(t)), "rg_get_histories")
        return s, t

    def set_histories(self, s=None, t=None):
        s = None if s is None else np.ascontiguousarray(s, np.float64)
        t = None if t is None else np.ascontiguousarray(t, np.float64)
        self._chk(self.L.rg_set_histories(self.h, _dp(s), _dp(t)), "rg_set_histories")

    def table_info(self):
        """(intervals per type pair, largest relative error) of the FP64
        pair-function tables; (0, 0.0) for analytic pair functions."""
        n = C.c_int()
        e = C.c_double()
        self._chk(self.L.rg_table_info(self.h, C.byref(n), C.byref(e)), "rg_table_info")
        return n.value, e.value

    def bond_table(self, bo_cut=0.3, max_per_atom=12):
        """Per-atom bonds with corrected BO > bo_cut (fix reax/c/bonds):
        (nbond[n], partner tags[n, max], bond orders[n, max], total BO[n],
        lone pairs[n]) in the original atom order."""
        nb = np.zeros(self.n, np.int32)
        tg = np.zeros((self.n, max_per_atom), np.int32)
        bo = np.zeros((self.n, max_per_atom))
        tot = np.zeros(self.n)
        nlp = np.zeros(self.n)
        rc = self.L.rg_bond_table(self.h, bo_cut, max_per_atom, _ip(nb), _ip(tg), _dp(bo),
                                  _dp(tot), _dp(nlp))
        self._chk(min(rc, 0), "rg_bond_table")
        return nb, tg, bo, tot, nlp

    def set_positions(self, x):
        x = np.ascontiguousarray(x, np.float64)
        self._chk(self.L.rg_set_positions(self.h, _dp(x)), "rg_set_positions")

    def qeq(self):
        q = np.zeros(self.n)
        a, b = C.c_int(), C.c_int()
        self._chk(self.L.rg_qeq(self.h, _dp(q), C.byref(a), C.byref(b)), "rg_qeq")
        return q, a.value, b.value

    def single_point(self, eflag=1, vflag=0):
        """QEq then the force step (rg_single_point: one graph launch once
        the same arrays were seen twice); returns q, f, energies."""
        q = np.zeros(self.n)
        f = np.zeros((self.n, 3))
        e = np.zeros(NENERGY)
        self._chk(self.L.rg_single_point(self.h, eflag, vflag, _dp(q), _dp(f), _dp(e)),
                  "rg_single_point")
        return q, f, dict(zip(ENERGY_NAMES, e))

    def compute(self, eflag=1, vflag=0):
        f = np.zeros((self.n, 3))
        e = np.zeros(NENERGY)
        self._chk(self.L.rg_compute(self.h, eflag, vflag, _dp(f), _dp(e)), "rg_compute")
        return f, dict(zip(ENERGY_NAMES, e))

    def virial(self):
        """Virial (xx, yy, zz, xy, xz, yz of sum r x f, kcal/mol) of the last
        force step computed with vflag, one row per segment."""
        ns = self.L.rg_num_segments(self.h)
        v = np.zeros((ns, 6))
        self._chk(self.L.rg_get_virial(self.h, _dp(v)), "rg_get_virial")
        return v

    def regroup(self, keep, src=None, sel=()):
        """Keep the segments `keep` (in that order) and append the segments
        `sel` of handle `src`, their state carried on the device; returns
        the new segments' first-atom offsets."""
        keep = np.ascontiguousarray(keep, np.int32)
        sel = np.ascontiguousarray(sel, np.int32)
        self._chk(self.L.rg_regroup_segments(self.h, len(keep), _ip(keep) if len(keep) else None,
                                             src.h if src is not None else None, len(sel),
                                             _ip(sel) if len(sel) else None),
                  "rg_regroup_segments")
        counts = [self._seg_counts[k] for k in keep] + \
                 ([src._seg_counts[k] for k in sel] if src is not None else [])
        self._seg_counts = counts
        self.nseg = len(counts)
        self.n = int(sum(counts))
        return np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(int)

    def segment_atoms(self, seg):
        """(x, v, q, f) of one segment."""
        c = self._seg_counts[seg]
        x = np.zeros((c, 3)); v = np.zeros((c, 3)); q = np.zeros(c); f = np.zeros((c, 3))
        self._chk(self.L.rg_get_segment_atoms(self.h, seg, _dp(x), _dp(v), _dp(q), _dp(f)),
                  "rg_get_segment_atoms")
        return x, v, q, f

    def atom_tallies(self):
        """Per-atom energy (n) and virial (n x 6: xx yy zz xy xz yz) of the
        last compute(eflag=3 or vflag=4), in the caller's atom order."""
        ea = np.zeros(self.n)
        va = np.zeros((self.n, 6))
        self._chk(self.L.rg_get_atom_tallies(self.h, _dp(ea), _dp(va)), "rg_get_atom_tallies")
        return ea, va

    def nve_initial(self, dt):
        self._chk(self.L.rg_nve_initial(self.h, dt), "rg_nve_initial")

    def nve_final(self, dt):
        self._chk(self.L.rg_nve_final(self.h, dt), "rg_nve_final")

    def run(self, nsteps, dt, energies=True):
        e = np.zeros(NENERGY) if energies else None
        self._chk(self.L.rg_run(self.h, nsteps, dt, _dp(e)), "rg_run")
        return dict(zip(ENERGY_NAMES, e)) if energies else None

    def set_state(self, x, v=None, f=None):
        """Positions (and optionally velocities and current forces) from host
        memory -- numpy arrays or raw pointers to pinned buffers -- keeping
        the QEq histories."""
        ptr = [a.ctypes.data if isinstance(a, np.ndarray) else a for a in (x, v, f)]
        self._chk(self.L.rg_set_state(self.h, *ptr), "rg_set_state")

    def get_atoms_into(self, x=None, v=None, q=None, f=None):
        """Copy the state into caller-provided host arrays (e.g. pinned)."""
        self._chk(self.L.rg_get_atoms(self.h, _dp(x), _dp(v), _dp(q), _dp(f)), "rg_get_atoms")

    def stream(self) -> int:
        return self.L.rg_stream(self.h)

    PHASES = ("bin_sort", "pair_list+H", "bond_list", "bond_orders", "atom_energy", "hbonds",
              "valence_torsion", "nonbonded", "dbond_forces", "force_out", "qeq_setup",
              "qeq_spmv", "qeq_vector", "qeq_finish", "nve")

    def profile(self, on: bool, phases=None):
        """Phase timing with CUDA events; phases (names of PHASES) limits
        the events to those phases (None: all)."""
        mask = 0xFFFFFFFF if phases is None else sum(1 << self.PHASES.index(p) for p in phases)
        self._chk(self.L.rg_profile_phases(self.h, mask), "rg_profile_phases")
        self._chk(self.L.rg_profile_enable(self.h, 1 if on else 0), "rg_profile_enable")

    def profile_get(self) -> dict:
        names = C.create_string_buffer(32 * 64)
        ms = np.zeros(64)
        cnt = np.zeros(64, np.int64)
        k = self.L.rg_profile_get(self.h, 64, names, _dp(ms),
                                  cnt.ctypes.data_as(C.POINTER(C.c_longlong)))
        out = {}
        for i in range(k):
            nm = names.raw[32 * i:32 * i + 32].split(b"\0")[0].decode()
            out[nm] = (float(ms[i]), int(cnt[i]))
        return out

    def get_atoms(self):
        n = self.n
        x, v, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        q = np.zeros(n)
        self._chk(self.L.rg_get_atoms(self.h, _dp(x), _dp(v), _dp(q), _dp(f)), "rg_get_atoms")
        return x, v, q, f

    def device_arrays(self):
        ptrs = [C.c_void_p() for _ in range(4)]
        self._chk(self.L.rg_device_arrays(self.h, *[C.byref(p) for p in ptrs]), "rg_device_arrays")
        return [p.value for p in ptrs]

    def stats(self):
        s = Stats()
        self._chk(self.L.rg_get_stats(self.h, C.byref(s)), "rg_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def synchronize(self):
        self._chk(self.L.rg_synchronize(self.h), "rg_synchronize")

    def _dump(self, fn, with_bo=False):
        k = fn(self.h, None, None, None, None) if with_bo else fn(self.h, None, None, None)
        if k < 0:
            raise ReaxError("list dump needs a preceding force step")
        ti, tj, im = (np.zeros(k, np.int32) for _ in range(3))
        if with_bo:
            bo = np.zeros((k, 4))
            fn(self.h, _ip(ti), _ip(tj), _ip(im), _dp(bo))
            return ti, tj, im, bo
        fn(self.h, _ip(ti), _ip(tj), _ip(im))
        return ti, tj, im

    def pair_list(self):
        return self._dump(self.L.rg_dump_pairs)

    def bond_list(self):
        return self._dump(self.L.rg_dump_bonds, True)

    def hbond_list(self):
        return self._dump(self.L.rg_dump_hbonds)
