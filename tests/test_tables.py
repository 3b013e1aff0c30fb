"""FP64 pair-function tables (cubic Hermite in r^2 of the vdW + Coulomb
energy and force factor and of the QEq H_ij, per type pair): built on the
host, checked against the analytic expressions at interior points of every
interval (no GPU needed)."""
import ctypes as C

from sw_reaxff_gb300 import api


def table_error(n, **kw):
    L = api.load_library()
    p = api.default_params(tabulate=n, **kw)
    e = C.c_double()
    assert L.rg_table_check(api.DEFAULT_FFIELD.encode(), C.byref(p), C.byref(e)) == 0
    return e.value


def test_default_tables_within_parity_bars():
    p = api.default_params()
    assert p.tabulate == 65536
    # relative to max(|f|, 1e-4 max|f|), far inside the 1e-9 parity bars
    assert table_error(p.tabulate) < 3e-10


def test_cubic_hermite_convergence():
    # fourth order: doubling the intervals divides the error by ~16
    e1, e2 = table_error(16384), table_error(32768)
    assert 8.0 < e1 / e2 < 24.0


def test_tables_follow_control():
    # a QEq taper radius beyond the nonbonded cutoff widens the tabulated
    # range; the tables stay accurate
    assert table_error(65536, qeq_swb=11.0) < 3e-10
