"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as
the checker or the timed CPU baseline; never by the product library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libreax_oracle.so")
# the reference's own host-side code + harness (built only where the
# reference sources exist: oracle/ref/Makefile)
REF_LIB = os.path.join(HERE, "_ref", "libreax_ref.so")

ENERGY_NAMES = ["e_bond", "e_ovun", "e_lp", "e_3", "e_ang", "e_pen", "e_coa",
                "e_hb", "e_tor", "e_con", "e_vdW", "e_ele", "e_12", "e_pol",
                "eng_vdwl", "eng_coul", "e_pol_phys"]
NENERGY = len(ENERGY_NAMES)


class Control(C.Structure):
    _fields_ = [("bond_cut", C.c_double), ("hbond_cut", C.c_double),
                ("thb_cut", C.c_double), ("thb_cutsq", C.c_double),
                ("skin", C.c_double), ("enobondsflag", C.c_int),
                ("lgflag", C.c_int), ("qeq_swa", C.c_double),
                ("qeq_swb", C.c_double), ("qeq_tol", C.c_double),
                ("qeq_imax", C.c_int)]


class Stats(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in (
        "n_local", "n_total", "n_far_local", "n_far_total", "n_bonds_total",
        "n_bonds_local", "n_hbonds", "n_H_entries")]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "reax_oracle.c")):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


_lib = None
_reflib = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def lib(path=None):
    global _lib, _reflib
    if path == REF_LIB:
        if _reflib is None:
            _reflib = _declare(C.CDLL(REF_LIB))
            P = C.POINTER
            _reflib.ro_ref_compute.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double),
                                               P(C.c_double), P(C.c_int), P(C.c_int),
                                               P(C.c_int), P(C.c_longlong)]
            _reflib.ro_ref_use_qeq.argtypes = [C.c_void_p, C.c_int]
            _reflib.ro_ref_atom_tallies.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        return _reflib
    if _lib is None:
        build()
        _lib = _declare(C.CDLL(LIB))
    return _lib


def _declare(L):
    if True:
        P = C.POINTER
        L.ro_default_control.argtypes = [P(Control)]
        L.ro_create.restype = C.c_void_p
        L.ro_create.argtypes = [C.c_char_p, P(Control), C.c_char_p, C.c_int]
        L.ro_destroy.argtypes = [C.c_void_p]
        L.ro_num_types.argtypes = [C.c_void_p]
        L.ro_type_param.restype = C.c_double
        L.ro_type_param.argtypes = [C.c_void_p, C.c_int, C.c_char_p]
        L.ro_set_system.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double),
                                    P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_double)]
        L.ro_set_tilt.argtypes = [C.c_void_p, P(C.c_double)]
        L.ro_qeq.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int), P(C.c_int)]
        L.ro_compute.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.ro_run_nve.argtypes = [C.c_void_p, C.c_int, C.c_double, P(C.c_double)]
        L.ro_md_steps.argtypes = [C.c_void_p, C.c_int, C.c_double, P(C.c_double)]
        L.ro_atom_tallies.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.ro_get_state.argtypes = [C.c_void_p] + [P(C.c_double)] * 4
        L.ro_get_stats.argtypes = [C.c_void_p, P(Stats)]
        for f in ("ro_dump_far", "ro_dump_hbonds"):
            getattr(L, f).restype = C.c_longlong
            getattr(L, f).argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int)]
        L.ro_dump_bonds.restype = C.c_longlong
        L.ro_dump_bonds.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int),
                                    P(C.c_double)]
        L.ro_dump_atom_terms.argtypes = [C.c_void_p, P(C.c_double)]
        L.ro_last_time.restype = C.c_double
        L.ro_last_time.argtypes = [C.c_void_p, C.c_int]
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


class Oracle:
    """Stateful CPU oracle for one periodic system."""

    def __init__(self, ffield: str, reference: bool = False, reference_qeq: bool = False,
                 **control):
        """reference=True loads the build that also carries the reference's
        own host-side code (ref_compute); reference_qeq=True (implies
        reference) makes qeq() and run_nve() solve the charges with the
        reference's own FixQEqReaxSunway::pre_force on this oracle's H
        matrix."""
        self.h = None
        L = lib(REF_LIB if (reference or reference_qeq) else None)
        ctl = Control()
        L.ro_default_control(C.byref(ctl))
        for k, v in control.items():
            setattr(ctl, k, v)
        err = C.create_string_buffer(512)
        self.h = L.ro_create(ffield.encode(), C.byref(ctl), err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        self.L = L
        self.n = 0
        if reference_qeq:
            L.ro_ref_use_qeq(self.h, 1)

    def close(self):
        if self.h:
            self.L.ro_destroy(self.h)
            self.h = None

    __del__ = close

    def type_param(self, t, what):
        return self.L.ro_type_param(self.h, t, what.encode())

    def set_system(self, box, x, types, tags=None, q=None, v=None, tilt=None):
        """tilt: (xy, xz, yz) of a triclinic cell, None for orthogonal."""
        self.L.ro_set_tilt(self.h, None if tilt is None else
                           _dp(np.ascontiguousarray(tilt, np.float64)))
        x = np.ascontiguousarray(x, np.float64)
        types = np.ascontiguousarray(types, np.int32)
        n = x.shape[0]
        box = np.ascontiguousarray(box, np.float64)
        tags = np.ascontiguousarray(tags if tags is not None else np.arange(1, n + 1), np.int32)
        q = None if q is None else np.ascontiguousarray(q, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        rc = self.L.ro_set_system(self.h, n, _dp(box), _dp(x), _ip(types), _ip(tags),
                                  _dp(q), _dp(v))
        if rc:
            raise ValueError("oracle rejected the system")
        self.n = n

    def qeq(self):
        q = np.zeros(self.n)
        its, itt = C.c_int(), C.c_int()
        self.L.ro_qeq(self.h, _dp(q), C.byref(its), C.byref(itt))
        return q, its.value, itt.value

    def compute(self):
        f = np.zeros((self.n, 3))
        e = np.zeros(NENERGY)
        self.L.ro_compute(self.h, _dp(f), _dp(e))
        return f, dict(zip(ENERGY_NAMES, e))

    def ref_compute(self):
        """The reference's own CPU routines on this oracle's lists: forces,
        energies, corrected bond orders (local bond entries in the oracle's
        order) and the reference-built H-bond list."""
        f = np.zeros((self.n, 3))
        e = np.zeros(NENERGY)
        nb = self.L.ro_dump_bonds(self.h, None, None, None, None)
        bo = np.zeros((max(nb, 1), 4))
        cap = max(self.stats()["n_far_local"], 1)
        ti = np.zeros(cap, np.int32); tj = np.zeros(cap, np.int32); im = np.zeros(cap, np.int32)
        nh = C.c_longlong()
        rc = self.L.ro_ref_compute(self.h, _dp(f), _dp(e), _dp(bo), _ip(ti), _ip(tj), _ip(im),
                                   C.byref(nh))
        if rc:
            raise RuntimeError(f"reference code aborted with {rc}")
        k = nh.value
        return f, dict(zip(ENERGY_NAMES, e)), bo[:nb], (ti[:k], tj[:k], im[:k])

    def atom_tallies(self, reference=False):
        """Per-atom energy (n) and virial (n x 6: xx yy zz xy xz yz) of the
        last compute (reference=True: of the last ref_compute, from the
        reference's own ev_tally_full)."""
        ea = np.zeros(self.n)
        va = np.zeros((self.n, 6))
        fn = self.L.ro_ref_atom_tallies if reference else self.L.ro_atom_tallies
        fn(self.h, _dp(ea), _dp(va))
        return ea, va

    def run_nve(self, nsteps, dt):
        e = np.zeros(NENERGY)
        self.L.ro_run_nve(self.h, nsteps, dt, _dp(e))
        return dict(zip(ENERGY_NAMES, e))

    def md_steps(self, nsteps, dt):
        """nsteps more NVE steps from the current state (after run_nve)."""
        e = np.zeros(NENERGY)
        self.L.ro_md_steps(self.h, nsteps, dt, _dp(e))
        return dict(zip(ENERGY_NAMES, e))

    def state(self):
        x = np.zeros((self.n, 3)); v = np.zeros((self.n, 3))
        q = np.zeros(self.n); f = np.zeros((self.n, 3))
        self.L.ro_get_state(self.h, _dp(x), _dp(v), _dp(q), _dp(f))
        return x, v, q, f

    def stats(self):
        s = Stats()
        self.L.ro_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def _dump(self, fn, with_bo=False):
        k = fn(self.h, None, None, None) if not with_bo else fn(self.h, None, None, None, None)
        ti = np.zeros(k, np.int32); tj = np.zeros(k, np.int32); im = np.zeros(k, np.int32)
        if with_bo:
            bo = np.zeros((k, 4))
            fn(self.h, _ip(ti), _ip(tj), _ip(im), _dp(bo))
            return ti, tj, im, bo
        fn(self.h, _ip(ti), _ip(tj), _ip(im))
        return ti, tj, im

    def far_list(self):
        return self._dump(self.L.ro_dump_far)

    def bond_list(self):
        return self._dump(self.L.ro_dump_bonds, True)

    def hbond_list(self):
        return self._dump(self.L.ro_dump_hbonds)

    def atom_terms(self):
        out = np.zeros((self.n, 8))
        self.L.ro_dump_atom_terms(self.h, _dp(out))
        return out

    def phase_times(self):
        return [self.L.ro_last_time(self.h, k) for k in range(6)]
