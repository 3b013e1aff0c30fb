/*
 * TEST INFRASTRUCTURE ONLY.  The few LAMMPS pieces that the reference's QEq
 * methods read, for one process without ghost atoms, so that the methods
 * themselves -- FixQEqReaxSunway::pre_force, init_matvec, CG_v2,
 * sparse_matvec and calculate_Q (fix_qeq_reax_sunway.cpp:539-600, 618-723,
 * 983-1167, 1573-1615, 1697-1755) -- compile unchanged from the reference
 * sources (oracle/ref/Makefile extracts them into oracle/_ref/src).
 *
 * The class below declares only the members those methods use, with the
 * names and types of fix_qeq_reax_sunway.h:37-150 (that is the interface
 * the extracted code is written against).  Communication is a no-op: the
 * matrix rows hold local atom indices (ghost images are folded onto their
 * owners), so no ghost copy of a vector exists.
 */
#ifndef RO_QEQ_SHIM_H
#define RO_QEQ_SHIM_H

#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mpi.h"
#include "gptl.h"
#include "reaxc_defs_sunway.h"
#include "reaxc_ctypes_sunway.h"

typedef int tagint;
typedef int64_t bigint;
#define BIGINT_FORMAT "%" PRId64
#define FLERR __FILE__, __LINE__

/* the reference's CPE entry points (fix_qeq_reax_sunway.cpp:45-51); defined
 * by ref_qeq.cpp for the host */
extern "C" {
void sparse_matvec_C(void *param);
void sparse_matvec_C_spawn(void *param);
void sparse_matvec_C_join();
void compute_H_Full_C(void *param);
}

namespace LAMMPS_NS {

struct NeighList {
  int inum = 0, gnum = 0;
  int *ilist = nullptr, *numneigh = nullptr;
  int **firstneigh = nullptr;
};

struct Atom {
  int nlocal = 0, nghost = 0, nmax = 0, ntypes = 0;
  int *type = nullptr, *mask = nullptr;
  tagint *tag = nullptr;
  double **x = nullptr;
  double *q = nullptr;
};

struct Comm {
  int me = 0;
  template <class F> void forward_comm_fix(F *) {}
  template <class F> void reverse_comm_fix(F *) {}
};

struct Update {
  bigint ntimestep = 0;
};

struct Error {
  int warnings = 0;
  void warning(const char *, int, const char *) { ++warnings; }
};

struct Memory {
  template <class T> T *create(T *&a, int n, const char *) {
    a = static_cast<T *>(calloc(n > 0 ? (size_t)n : 1, sizeof(T)));
    return a;
  }
  template <class T> void destroy(T *&a) {
    free(a);
    a = nullptr;
  }
};

struct PairReaxCSunway {
  NeighList *listfull = nullptr;
};

class FixQEqReaxSunway {
 public:
  /* LAMMPS Pointers / Fix members */
  Atom *atom = nullptr;
  Comm *comm = nullptr;
  Update *update = nullptr;
  Error *error = nullptr;
  Memory *memory = nullptr;
  MPI_Comm world = 0;
  int groupbit = 1;

  /* FixQEqReaxSunway members (fix_qeq_reax_sunway.h) */
  int matvecs = 0;
  double qeq_time = 0;
  int nevery = 1;
  int n = 0, N = 0, m_fill = 0;
  int n_cap = 0, nmax = 0, m_cap = 0;
  int pack_flag = 0;
  NeighList *list = nullptr;
  PairReaxCSunway *reaxc = nullptr;
  double *m = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *z = nullptr,
         *ss = nullptr, *n_test = nullptr;
  double swa = 0, swb = 10;
  double Tap[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  double tolerance = 1e-6;
  double *chi = nullptr, *eta = nullptr, *gamma = nullptr;
  double **shld = nullptr;
  double *s = nullptr, *t = nullptr;
  double **s_hist = nullptr, **t_hist = nullptr;
  int nprev = 5;
  typedef struct {
    int n, m;
    int *firstnbr;
    int *numnbrs;
    int *jlist;
    double *val;
  } sparse_matrix;
  sparse_matrix H;
  double *Hdia_inv = nullptr;
  double *b_s = nullptr, *b_t = nullptr;
  int maxHlist = 0;
  double *p = nullptr, *q = nullptr, *r = nullptr, *d = nullptr;
  int dual_enabled = 0;
  int matvecs_s = 0, matvecs_t = 0;

  /* storage is sized by the harness before the first call */
  void reallocate_storage() {}
  void reallocate_matrix() {}

  /* the reference's own methods (extracted) */
  void pre_force(int);
  void init_matvec();
  int CG_v2(double *, double *);
  void sparse_matvec(sparse_matrix *, double *, double *);
  void calculate_Q();
};

}  // namespace LAMMPS_NS

#endif
