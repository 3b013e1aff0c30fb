/*
 * TEST INFRASTRUCTURE ONLY (built by oracle/ref/Makefile where the reference
 * sources are present).  Runs the reference's own QEq driver -- the methods
 * FixQEqReaxSunway::pre_force, init_matvec, CG_v2, sparse_matvec and
 * calculate_Q, compiled unchanged from fix_qeq_reax_sunway.cpp against
 * qeq_shim.h -- on a matrix built by the oracle, so that the oracle's
 * restatement of the pipelined CG, the s/t extrapolation and the charge
 * split (reax_oracle.c ro_qeq) is checked against the reference's code.
 *
 * What stays restated here: the two CPE kernels those methods call.
 *  - compute_H_Full_C (fix_qeq_reax_sw64.c:75-295, CPE body :768-911) fills
 *    the H rows; the harness hands the methods a matrix the oracle already
 *    built from the same formula (reax_oracle.c ro_qeq), so it is a no-op.
 *  - sparse_matvec_C / _spawn / _join (fix_qeq_reax_sw64.c:42-73, CPE body
 *    sparse_matvec_C_para :357-498): b_i = eta_{type i} x_i, then
 *    b_i += H_ij x_j in row order -- the CPE kernel's order, which is also
 *    the reference's dead host loop (fix_qeq_reax_sunway.cpp:1597-1615).  A
 *    spawned product runs to completion at the spawn: in CG_v2 the host
 *    work between spawn and join neither reads q nor writes d, so the
 *    result is the same as the overlapped one.
 */
#include <climits>
#include <vector>

#include "qeq_shim.h"

#ifndef SQR
#define SQR(x) ((x) * (x))
#endif
#ifndef CUBE
#define CUBE(x) ((x) * (x) * (x))
#endif
#ifndef EV_TO_KCAL_PER_MOL
#define EV_TO_KCAL_PER_MOL 14.4
#endif

using namespace LAMMPS_NS;

#include "fix_qeq_methods.inc"

extern "C" void compute_H_Full_C(void *) {}

extern "C" void sparse_matvec_C(void *param) {
  const fix_qeq_pack_t *pm = static_cast<const fix_qeq_pack_t *>(param);
  for (int ii = 0; ii < pm->list.inum; ++ii) {
    const int i = pm->list.ilist[ii];
    if (pm->atom.mask[i] & pm->groupbit) pm->b[i] = pm->eta[pm->atom.type[i]] * pm->x[i];
    const int e = pm->H.firstnbr[i] + pm->H.numnbrs[i];
    for (int k = pm->H.firstnbr[i]; k < e; ++k) pm->b[i] += pm->H.val[k] * pm->x[pm->H.jlist[k]];
  }
}

extern "C" void sparse_matvec_C_spawn(void *param) { sparse_matvec_C(param); }
extern "C" void sparse_matvec_C_join() {}

/* One FixQEqReaxSunway::pre_force on n local atoms.  type[i] indexes the
 * per-type chi/eta arrays; the matrix is CSR (start[n+1], col, val) with
 * local column indices; s_hist/t_hist are n x 5 row-major and are updated in
 * place, like s, t (length n) and q_out.  Returns the number of CG
 * non-convergence warnings the methods raised. */
extern "C" int ref_qeq_pre_force(int n, const int *type, int ntypes, const double *chi,
                                 const double *eta, const int *start, const int *col,
                                 const double *val, double tol, double *s_hist, double *t_hist,
                                 double *s, double *t, double *q_out, int *iters_s,
                                 int *iters_t) {
  std::vector<int> mask(n, 1), ilist(n), numnbrs(n), first(n);
  std::vector<double *> sh(n), th(n);
  std::vector<double> Hdia_inv(n), b_s(n), b_t(n), p(n), q(n), r(n), d(n);
  /* atom->x is only repacked into the (unused) H-build pack by init_matvec */
  std::vector<double> xs(3 * (size_t)n + 3);
  std::vector<double *> xrow(n + 1);
  for (int i = 0; i <= n; ++i) xrow[i] = xs.data() + 3 * (size_t)i;
  for (int i = 0; i < n; ++i) {
    ilist[i] = i;
    first[i] = start[i];
    numnbrs[i] = start[i + 1] - start[i];
    sh[i] = s_hist + 5 * (size_t)i;
    th[i] = t_hist + 5 * (size_t)i;
  }
  Atom atom;
  atom.nlocal = n;
  atom.nmax = n;
  atom.ntypes = ntypes;
  atom.type = const_cast<int *>(type);
  atom.mask = mask.data();
  atom.q = q_out;
  atom.x = xrow.data();
  NeighList full;
  full.inum = n;
  full.ilist = ilist.data();
  PairReaxCSunway pair;
  pair.listfull = &full;
  Comm comm;
  Update update;
  Error error;
  Memory memory;

  FixQEqReaxSunway fx;
  fx.atom = &atom;
  fx.comm = &comm;
  fx.update = &update;
  fx.error = &error;
  fx.memory = &memory;
  fx.reaxc = &pair;
  fx.list = &full;
  fx.nmax = n;
  fx.n_cap = INT_MAX / 2;
  fx.m_cap = INT_MAX / 2;
  fx.tolerance = tol;
  fx.chi = const_cast<double *>(chi);
  fx.eta = const_cast<double *>(eta);
  fx.s = s;
  fx.t = t;
  fx.s_hist = sh.data();
  fx.t_hist = th.data();
  fx.H.n = n;
  fx.H.m = start[n];
  fx.H.firstnbr = first.data();
  fx.H.numnbrs = numnbrs.data();
  fx.H.jlist = const_cast<int *>(col);
  fx.H.val = const_cast<double *>(val);
  fx.Hdia_inv = Hdia_inv.data();
  fx.b_s = b_s.data();
  fx.b_t = b_t.data();
  fx.p = p.data();
  fx.q = q.data();
  fx.r = r.data();
  fx.d = d.data();

  fx.pre_force(0);

  if (iters_s) *iters_s = fx.matvecs_s;
  if (iters_t) *iters_t = fx.matvecs_t;
  return error.warnings;
}
