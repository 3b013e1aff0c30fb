/*
 * CPU oracle for the ReaxFF force step -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement (own code) of the SW_REAXFF reference CPU path.  Each
 * routine names the reference file:line it follows.  Parity of this oracle
 * is pinned against the reference's own compiled host code in
 * oracle/ref_harness.c (built only where the reference sources exist).
 *
 * Floating-point contract: build with -ffp-contract=off so that distances
 * (d^2 = dx*dx + dy*dy + dz*dz, left to right) round exactly like the CUDA
 * path's non-contracted membership tests.
 */
#include "reax_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define MAXT 8
#define MAX_3BODY 5
#define SQR(x) ((x) * (x))
#define CUBE(x) ((x) * (x) * (x))
/* constants of reaxc_defs_sunway.h:58-69 */
#define constPI 3.14159265
#define DEG2RAD(a) ((a)*constPI / 180.0)
#define C_ele 332.06371
#define KCALpMOL_to_EV 23.02
#define EV_TO_KCAL_PER_MOL 14.4
#define HB_THRESHOLD 1e-2
#define MIN_SINE 1e-10
/* LAMMPS real units: ftm2v = 1/48.88821291^2 (force*time/mass -> velocity) */
#define FTM2V (1.0 / 48.88821291 / 48.88821291)

typedef struct {
  char name[16];
  double r_s, valency, mass, r_vdw, epsilon, gamma, r_pi, valency_e, nlp_opt;
  double alpha, gamma_w, valency_boc, p_ovun5, chi, eta;
  int p_hbond;
  double r_pi_pi, p_lp2, b_o_131, b_o_132, b_o_133;
  double p_ovun2, p_val3, valency_val, p_val5, rcore2, ecore2, acore2;
  double lgcij, lgre;
} sbp_t;

typedef struct {
  double r_s, r_p, r_pp, p_bo1, p_bo2, p_bo3, p_bo4, p_bo5, p_bo6;
  double p_boc3, p_boc4, p_boc5, v13cor, ovc;
  double De_s, De_p, De_pp, p_be1, p_be2, p_ovun1;
  double D, alpha, r_vdW, gamma_w, gamma, rcore, ecore, acore, lgcij, lgre;
} tbp_t;

typedef struct {
  double theta_00, p_val1, p_val2, p_coa1, p_val7, p_pen1, p_val4;
} thbp_t;
typedef struct {
  int cnt;
  thbp_t prm[MAX_3BODY];
} thbh_t;
typedef struct {
  double V1, V2, V3, p_tor1, p_cot1;
} fbp_t;
typedef struct {
  int cnt;
  fbp_t prm;
} fbh_t;
typedef struct {
  double r0_hb, p_hb1, p_hb2, p_hb3;
} hbp_t;

typedef struct {
  int ntypes;
  double gp[64];
  int ngp;
  int vdw_type;
  sbp_t sbp[MAXT];
  tbp_t tbp[MAXT][MAXT];
  thbh_t thbp[MAXT][MAXT][MAXT];
  hbp_t hbp[MAXT][MAXT][MAXT];
  fbh_t fbp[MAXT][MAXT][MAXT][MAXT];
} ffield_t;

/* one entry of the bond list (bond_data + bond_order_data + the SoA lists
 * BO_list / BOpi_list / Cdbo*_list of reaxc_ctypes_sunway.h:612-651) */
typedef struct {
  int nbr, sym, far;
  double d, dvec[3];
  double BO, BO_s, BO_pi, BO_pi2;
  double dBOp[3], dln_BOp_s[3], dln_BOp_pi[3], dln_BOp_pi2[3];
  double C1dbo, C2dbo, C3dbo;
  double C1dbopi, C2dbopi, C3dbopi, C4dbopi;
  double C1dbopi2, C2dbopi2, C3dbopi2, C4dbopi2;
  double Cdbo, Cdbopi, Cdbopi2;
} bond_t;

struct ro_ctx {
  ffield_t ff;
  ro_control ctl;
  double bo_cut, nonb_cut, nonb_low;
  double Tap[8];     /* pair taper, Init_Taper reaxc_init_md_sunway.cpp:100 */
  double qTap[8];    /* QEq taper, init_taper fix_qeq_reax_sunway.cpp:458 */
  double L[3];
  double T[3];       /* tilts xy, xz, yz (0: orthogonal) */
  int tri;
  /* local atoms */
  int n;
  double *x, *v, *q, *f;
  int *type, *tag;
  double *s_hist, *t_hist; /* [n*5] */
  double *s, *t;
  /* extended (local + ghost) */
  int N, capN;
  double *xe;
  int *te, *own, *imgc;
  /* far list (full) */
  int *far_start;
  int *far_nbr;
  double *far_d, *far_dvec;
  long long far_cap;
  /* bonds */
  int *b_start, *b_end;
  bond_t *bonds;
  long long bond_cap;
  /* hbonds (local H atoms): far-list entry indices */
  int *hb_start;
  int *hb_far;
  long long hb_cap;
  /* per-atom workspace over N */
  double *bo_dboc0, *bo_dboc1, *Deltap, *Deltap_boc, *Delta, *Delta_e,
      *Delta_val, *vlpex, *nlp, *nlp_temp, *Delta_lp, *Delta_lp_temp,
      *dDelta_lp, *dDelta_lp_temp, *Clp;
  double *dDeltap_self; /* 3N */
  double *fC;           /* 4N: force[0..2] + CdDelta[3] */
  double *cd_local;     /* n: folded CdDelta */
  /* QEq matrix rows for local atoms */
  long long H_entries;
  /* per-atom nonbonded tallies of the last ro_compute (ev_tally_full):
   * eatom[n], vatom[6n] (xx yy zz xy xz yz per atom); the reference build
   * keeps the reference's own in ref_eatom / ref_vatom */
  double *eatom, *vatom, *ref_eatom, *ref_vatom;
  int tally_n;
  /* QEq driver: NULL = qeq_restated below; the reference build installs the
   * reference's own FixQEqReaxSunway::pre_force here (oracle/ref) */
  int (*qeq_driver)(ro_ctx *c, const void *H, int *iters_s, int *iters_t);
  double en[RO_NENERGY];
  double tphase[8];
};

/* ------------------------------------------------------------------ */
/* force-field reader: restates Read_Force_Field,
 * reaxc_ffield_sunway.cpp:35-714 */

static int tokenize(char *s, char **tok, int maxtok) {
  int c = 0;
  char *p = strtok(s, " \t\n\r!");
  while (p && c < maxtok) {
    tok[c++] = p;
    p = strtok(NULL, " \t\n\r!");
  }
  return c;
}

static int read_ffield(const char *path, ffield_t *ff, int lgflag,
                       char *err, int errlen) {
  FILE *fp = fopen(path, "r");
  char line[1024], *tok[64];
  int i, j, k, m, n, c, l;
  if (!fp) {
    snprintf(err, errlen, "cannot open force field %s", path);
    return -1;
  }
  memset(ff, 0, sizeof(*ff));
#define RD()                                                  \
  do {                                                        \
    if (!fgets(line, sizeof line, fp)) {                      \
      snprintf(err, errlen, "premature end of force field");  \
      fclose(fp);                                             \
      return -1;                                              \
    }                                                         \
    c = tokenize(line, tok, 64);                              \
  } while (0)
  RD(); /* header comment */
  RD();
  n = atoi(tok[0]);
  if (n < 1 || n > 64) {
    snprintf(err, errlen, "bad number of global parameters %d", n);
    fclose(fp);
    return -1;
  }
  ff->ngp = n;
  for (i = 0; i < n; i++) {
    RD();
    ff->gp[i] = atof(tok[0]);
  }
  RD();
  ff->ntypes = atoi(tok[0]);
  if (ff->ntypes < 1 || ff->ntypes > MAXT) {
    snprintf(err, errlen, "unsupported number of atom types %d", ff->ntypes);
    fclose(fp);
    return -1;
  }
  RD(); RD(); RD();
  ff->vdw_type = 0;
  for (i = 0; i < ff->ntypes; i++) {
    sbp_t *s = &ff->sbp[i];
    RD();
    for (j = 0; j < (int)strlen(tok[0]) && j < 15; j++)
      s->name[j] = (char)toupper((unsigned char)tok[0][j]);
    s->r_s = atof(tok[1]); s->valency = atof(tok[2]); s->mass = atof(tok[3]);
    s->r_vdw = atof(tok[4]); s->epsilon = atof(tok[5]); s->gamma = atof(tok[6]);
    s->r_pi = atof(tok[7]); s->valency_e = atof(tok[8]);
    s->nlp_opt = 0.5 * (s->valency_e - s->valency);
    RD();
    s->alpha = atof(tok[0]); s->gamma_w = atof(tok[1]);
    s->valency_boc = atof(tok[2]); s->p_ovun5 = atof(tok[3]);
    s->chi = atof(tok[5]); s->eta = 2.0 * atof(tok[6]);
    s->p_hbond = (int)atof(tok[7]);
    RD();
    s->r_pi_pi = atof(tok[0]); s->p_lp2 = atof(tok[1]);
    s->b_o_131 = atof(tok[3]); s->b_o_132 = atof(tok[4]);
    s->b_o_133 = atof(tok[5]);
    RD();
    if (c < 3) {
      snprintf(err, errlen, "inconsistent ffield file");
      fclose(fp);
      return -1;
    }
    s->p_ovun2 = atof(tok[0]); s->p_val3 = atof(tok[1]);
    s->valency_val = atof(tok[3]); s->p_val5 = atof(tok[4]);
    s->rcore2 = atof(tok[5]); s->ecore2 = atof(tok[6]); s->acore2 = atof(tok[7]);
    if (lgflag) {
      RD();
      s->lgcij = atof(tok[0]); s->lgre = atof(tok[1]);
    }
    /* vdW type selection, reaxc_ffield_sunway.cpp:229-284 */
    if (s->rcore2 > 0.01 && s->acore2 > 0.01) {
      if (s->gamma_w > 0.5) {
        if (ff->vdw_type == 0 || ff->vdw_type == 3) ff->vdw_type = 3;
      } else {
        if (ff->vdw_type == 0 || ff->vdw_type == 2) ff->vdw_type = 2;
      }
    } else {
      if (s->gamma_w > 0.5) {
        if (ff->vdw_type == 0 || ff->vdw_type == 1) ff->vdw_type = 1;
      } else {
        snprintf(err, errlen, "no shielding or inner wall for element %s",
                 s->name);
        fclose(fp);
        return -1;
      }
    }
  }
  for (i = 0; i < ff->ntypes; i++)
    if (ff->sbp[i].mass < 21 &&
        ff->sbp[i].valency_val != ff->sbp[i].valency_boc)
      ff->sbp[i].valency_val = ff->sbp[i].valency_boc;
  /* two-body */
  RD();
  l = atoi(tok[0]);
  RD();
  for (i = 0; i < l; i++) {
    RD();
    j = atoi(tok[0]) - 1;
    k = atoi(tok[1]) - 1;
    double v[10];
    for (m = 0; m < 8; m++) v[m] = atof(tok[2 + m]);
    RD();
    if (j < ff->ntypes && k < ff->ntypes && j >= 0 && k >= 0) {
      tbp_t *a = &ff->tbp[j][k], *b = &ff->tbp[k][j];
      a->De_s = b->De_s = v[0]; a->De_p = b->De_p = v[1];
      a->De_pp = b->De_pp = v[2]; a->p_be1 = b->p_be1 = v[3];
      a->p_bo5 = b->p_bo5 = v[4]; a->v13cor = b->v13cor = v[5];
      a->p_bo6 = b->p_bo6 = v[6]; a->p_ovun1 = b->p_ovun1 = v[7];
      a->p_be2 = b->p_be2 = atof(tok[0]); a->p_bo3 = b->p_bo3 = atof(tok[1]);
      a->p_bo4 = b->p_bo4 = atof(tok[2]); a->p_bo1 = b->p_bo1 = atof(tok[4]);
      a->p_bo2 = b->p_bo2 = atof(tok[5]); a->ovc = b->ovc = atof(tok[6]);
    }
  }
  for (i = 0; i < ff->ntypes; i++)
    for (j = i; j < ff->ntypes; j++) {
      sbp_t *si = &ff->sbp[i], *sj = &ff->sbp[j];
      tbp_t *a = &ff->tbp[i][j], *b = &ff->tbp[j][i];
      a->r_s = 0.5 * (si->r_s + sj->r_s); b->r_s = 0.5 * (sj->r_s + si->r_s);
      a->r_p = 0.5 * (si->r_pi + sj->r_pi); b->r_p = 0.5 * (sj->r_pi + si->r_pi);
      a->r_pp = 0.5 * (si->r_pi_pi + sj->r_pi_pi);
      b->r_pp = 0.5 * (sj->r_pi_pi + si->r_pi_pi);
      a->p_boc3 = sqrt(si->b_o_132 * sj->b_o_132);
      b->p_boc3 = sqrt(sj->b_o_132 * si->b_o_132);
      a->p_boc4 = sqrt(si->b_o_131 * sj->b_o_131);
      b->p_boc4 = sqrt(sj->b_o_131 * si->b_o_131);
      a->p_boc5 = sqrt(si->b_o_133 * sj->b_o_133);
      b->p_boc5 = sqrt(sj->b_o_133 * si->b_o_133);
      a->D = sqrt(si->epsilon * sj->epsilon);
      b->D = sqrt(sj->epsilon * si->epsilon);
      a->alpha = sqrt(si->alpha * sj->alpha);
      b->alpha = sqrt(sj->alpha * si->alpha);
      a->r_vdW = 2.0 * sqrt(si->r_vdw * sj->r_vdw);
      b->r_vdW = 2.0 * sqrt(sj->r_vdw * si->r_vdw);
      a->gamma_w = sqrt(si->gamma_w * sj->gamma_w);
      b->gamma_w = sqrt(sj->gamma_w * si->gamma_w);
      a->gamma = pow(si->gamma * sj->gamma, -1.5);
      b->gamma = pow(sj->gamma * si->gamma, -1.5);
      a->rcore = b->rcore = sqrt(si->rcore2 * sj->rcore2);
      a->ecore = b->ecore = sqrt(si->ecore2 * sj->ecore2);
      a->acore = b->acore = sqrt(si->acore2 * sj->acore2);
      a->lgcij = b->lgcij = sqrt(si->lgcij * sj->lgcij);
      a->lgre = b->lgre = 2.0 * ff->gp[35] * sqrt(si->lgre * sj->lgre);
    }
  /* off-diagonal */
  RD();
  l = atoi(tok[0]);
  for (i = 0; i < l; i++) {
    RD();
    j = atoi(tok[0]) - 1;
    k = atoi(tok[1]) - 1;
    if (j < ff->ntypes && k < ff->ntypes && j >= 0 && k >= 0) {
      tbp_t *a = &ff->tbp[j][k], *b = &ff->tbp[k][j];
      double val;
      val = atof(tok[2]); if (val > 0.0) a->D = b->D = val;
      val = atof(tok[3]); if (val > 0.0) a->r_vdW = b->r_vdW = 2 * val;
      val = atof(tok[4]); if (val > 0.0) a->alpha = b->alpha = val;
      val = atof(tok[5]); if (val > 0.0) a->r_s = b->r_s = val;
      val = atof(tok[6]); if (val > 0.0) a->r_p = b->r_p = val;
      val = atof(tok[7]); if (val > 0.0) a->r_pp = b->r_pp = val;
      if (c > 8) { val = atof(tok[8]); if (val >= 0.0) a->lgcij = b->lgcij = val; }
    }
  }
  /* three-body */
  RD();
  l = atoi(tok[0]);
  for (i = 0; i < l; i++) {
    RD();
    j = atoi(tok[0]) - 1;
    k = atoi(tok[1]) - 1;
    m = atoi(tok[2]) - 1;
    if (j < ff->ntypes && k < ff->ntypes && m < ff->ntypes && j >= 0 &&
        k >= 0 && m >= 0) {
      int cnt = ff->thbp[j][k][m].cnt;
      if (cnt >= MAX_3BODY - 1) continue;
      /* both counters advance, also when j == m (the second slot then
       * stays zero and is skipped by the |p_val1| > 0.001 test), as in
       * reaxc_ffield_sunway.cpp:560-563 */
      ff->thbp[j][k][m].cnt++;
      ff->thbp[m][k][j].cnt++;
      thbp_t p;
      p.theta_00 = atof(tok[3]); p.p_val1 = atof(tok[4]);
      p.p_val2 = atof(tok[5]); p.p_coa1 = atof(tok[6]);
      p.p_val7 = atof(tok[7]); p.p_pen1 = atof(tok[8]);
      p.p_val4 = atof(tok[9]);
      ff->thbp[j][k][m].prm[cnt] = p;
      ff->thbp[m][k][j].prm[cnt] = p;
    }
  }
  /* four-body */
  {
    static char tor_flag[MAXT][MAXT][MAXT][MAXT];
    memset(tor_flag, 0, sizeof tor_flag);
    RD();
    l = atoi(tok[0]);
    for (i = 0; i < l; i++) {
      RD();
      j = atoi(tok[0]) - 1;
      k = atoi(tok[1]) - 1;
      m = atoi(tok[2]) - 1;
      n = atoi(tok[3]) - 1;
      fbp_t p;
      p.V1 = atof(tok[4]); p.V2 = atof(tok[5]); p.V3 = atof(tok[6]);
      p.p_tor1 = atof(tok[7]); p.p_cot1 = atof(tok[8]);
      if (j >= 0 && n >= 0) {
        if (j < ff->ntypes && k < ff->ntypes && m < ff->ntypes &&
            n < ff->ntypes) {
          tor_flag[j][k][m][n] = tor_flag[n][m][k][j] = 1;
          ff->fbp[j][k][m][n].cnt = ff->fbp[n][m][k][j].cnt = 1;
          ff->fbp[j][k][m][n].prm = p;
          ff->fbp[n][m][k][j].prm = p;
        }
      } else if (k < ff->ntypes && m < ff->ntypes && k >= 0 && m >= 0) {
        int p1, o;
        for (p1 = 0; p1 < ff->ntypes; p1++)
          for (o = 0; o < ff->ntypes; o++) {
            ff->fbp[p1][k][m][o].cnt = 1;
            ff->fbp[o][m][k][p1].cnt = 1;
            if (!tor_flag[p1][k][m][o]) ff->fbp[p1][k][m][o].prm = p;
            if (!tor_flag[o][m][k][p1]) ff->fbp[o][m][k][p1].prm = p;
          }
      }
    }
  }
  /* hydrogen bonds */
  for (i = 0; i < ff->ntypes; i++)
    for (j = 0; j < ff->ntypes; j++)
      for (k = 0; k < ff->ntypes; k++) ff->hbp[i][j][k].r0_hb = -1.0;
  RD();
  l = atoi(tok[0]);
  for (i = 0; i < l; i++) {
    if (!fgets(line, sizeof line, fp)) break;
    c = tokenize(line, tok, 64);
    if (c < 7) continue;
    j = atoi(tok[0]) - 1;
    k = atoi(tok[1]) - 1;
    m = atoi(tok[2]) - 1;
    if (j < ff->ntypes && m < ff->ntypes && j >= 0 && k >= 0 && m >= 0 &&
        k < ff->ntypes) {
      ff->hbp[j][k][m].r0_hb = atof(tok[3]);
      ff->hbp[j][k][m].p_hb1 = atof(tok[4]);
      ff->hbp[j][k][m].p_hb2 = atof(tok[5]);
      ff->hbp[j][k][m].p_hb3 = atof(tok[6]);
    }
  }
#undef RD
  fclose(fp);
  return 0;
}

/* Init_Taper, reaxc_init_md_sunway.cpp:100-136 (same polynomial as the
 * QEq fix's init_taper, fix_qeq_reax_sunway.cpp:458-484) */
static void init_taper(double swa, double swb, double *Tap) {
  double d7 = pow(swb - swa, 7.0);
  double swa2 = SQR(swa), swa3 = CUBE(swa), swb2 = SQR(swb), swb3 = CUBE(swb);
  Tap[7] = 20.0 / d7;
  Tap[6] = -70.0 * (swa + swb) / d7;
  Tap[5] = 84.0 * (swa2 + 3.0 * swa * swb + swb2) / d7;
  Tap[4] = -35.0 * (swa3 + 9.0 * swa2 * swb + 9.0 * swa * swb2 + swb3) / d7;
  Tap[3] = 140.0 * (swa3 * swb + 3.0 * swa2 * swb2 + swa * swb3) / d7;
  Tap[2] = -210.0 * (swa3 * swb2 + swa2 * swb3) / d7;
  Tap[1] = 140.0 * swa3 * swb3 / d7;
  Tap[0] = (-35.0 * swa3 * swb2 * swb2 + 21.0 * swa2 * swb3 * swb2 +
            7.0 * swa * swb3 * swb3 + swb3 * swb3 * swb) / d7;
}

void ro_default_control(ro_control *c) {
  c->bond_cut = 5.0;
  c->hbond_cut = 7.5;
  c->thb_cut = 0.001;
  c->thb_cutsq = 0.00001;
  c->skin = 2.5;
  c->enobondsflag = 1;
  c->lgflag = 0;
  c->qeq_swa = 0.0;
  c->qeq_swb = 10.0;
  c->qeq_tol = 1e-6;
  c->qeq_imax = 200;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

ro_ctx *ro_create(const char *path, const ro_control *ctl, char *err,
                  int errlen) {
  ro_ctx *c = (ro_ctx *)calloc(1, sizeof(ro_ctx));
  char dummy[256];
  if (!err) { err = dummy; errlen = sizeof dummy; }
  if (ctl) c->ctl = *ctl; else ro_default_control(&c->ctl);
  if (read_ffield(path, &c->ff, c->ctl.lgflag, err, errlen)) {
    free(c);
    return NULL;
  }
  /* reaxc_ffield_sunway.cpp:86-88 */
  c->bo_cut = 0.01 * c->ff.gp[29];
  c->nonb_low = c->ff.gp[11];
  c->nonb_cut = c->ff.gp[12];
  init_taper(c->nonb_low, c->nonb_cut, c->Tap);
  init_taper(c->ctl.qeq_swa, c->ctl.qeq_swb, c->qTap);
  return c;
}

static void free_work(ro_ctx *c) {
  free(c->xe); free(c->te); free(c->own); free(c->imgc);
  free(c->far_start); free(c->far_nbr); free(c->far_d); free(c->far_dvec);
  free(c->b_start); free(c->b_end); free(c->bonds);
  free(c->hb_start); free(c->hb_far);
  free(c->bo_dboc0); free(c->bo_dboc1); free(c->Deltap); free(c->Deltap_boc);
  free(c->Delta); free(c->Delta_e); free(c->Delta_val); free(c->vlpex);
  free(c->nlp); free(c->nlp_temp); free(c->Delta_lp); free(c->Delta_lp_temp);
  free(c->dDelta_lp); free(c->dDelta_lp_temp); free(c->Clp);
  free(c->dDeltap_self); free(c->fC);
  c->xe = c->far_d = c->far_dvec = NULL;
  c->te = c->own = c->imgc = c->far_start = c->far_nbr = NULL;
  c->b_start = c->b_end = c->hb_start = c->hb_far = NULL;
  c->bonds = NULL;
  c->bo_dboc0 = c->bo_dboc1 = c->Deltap = c->Deltap_boc = c->Delta = NULL;
  c->Delta_e = c->Delta_val = c->vlpex = c->nlp = c->nlp_temp = NULL;
  c->Delta_lp = c->Delta_lp_temp = c->dDelta_lp = c->dDelta_lp_temp = NULL;
  c->Clp = c->dDeltap_self = c->fC = NULL;
  c->capN = 0;
  c->far_cap = c->bond_cap = c->hb_cap = 0;
}

void ro_destroy(ro_ctx *c) {
  if (!c) return;
  free_work(c);
  free(c->x); free(c->v); free(c->q); free(c->f); free(c->type); free(c->tag);
  free(c->s_hist); free(c->t_hist); free(c->s); free(c->t); free(c->cd_local);
  free(c->eatom); free(c->vatom); free(c->ref_eatom); free(c->ref_vatom);
  free(c);
}

int ro_num_types(const ro_ctx *c) { return c->ff.ntypes; }
double ro_global_param(const ro_ctx *c, int idx) {
  return (idx >= 0 && idx < c->ff.ngp) ? c->ff.gp[idx] : 0.0;
}
double ro_type_param(const ro_ctx *c, int t, const char *what) {
  if (t < 0 || t >= c->ff.ntypes) return 0.0;
  const sbp_t *s = &c->ff.sbp[t];
  if (!strcmp(what, "mass")) return s->mass;
  if (!strcmp(what, "chi")) return s->chi;
  if (!strcmp(what, "eta")) return s->eta;
  if (!strcmp(what, "gamma")) return s->gamma;
  if (!strcmp(what, "p_hbond")) return s->p_hbond;
  return 0.0;
}

static double wrap1(double x, double L) {
  double y = x - L * floor(x / L);
  if (y >= L) y -= L;
  if (y < 0) y = 0;
  return y;
}

/* Triclinic cell (LAMMPS's restricted form: a = (lx,0,0), b = (xy,ly,0),
 * c = (xz,yz,lz)); LAMMPS's Domain/Comm give the reference these images as
 * ghost atoms.  Fractional coordinates by back-substitution and the wrap by
 * the lattice translation floor(fractional), each operation rounded once
 * (the device code does the same). */
static void frac3(const ro_ctx *c, const double *x, double *u) {
  u[2] = x[2] / c->L[2];
  u[1] = (x[1] - u[2] * c->T[2]) / c->L[1];
  u[0] = ((x[0] - u[1] * c->T[0]) - u[2] * c->T[1]) / c->L[0];
}

static void img_vec(const ro_ctx *c, int sx, int sy, int sz, double *v) {
  v[0] = ((double)sx * c->L[0] + (double)sy * c->T[0]) + (double)sz * c->T[1];
  v[1] = (double)sy * c->L[1] + (double)sz * c->T[2];
  v[2] = (double)sz * c->L[2];
}

static void wrap_pos(const ro_ctx *c, double *x) {
  int d;
  if (!c->tri) {
    for (d = 0; d < 3; d++) x[d] = wrap1(x[d], c->L[d]);
    return;
  }
  double u[3];
  frac3(c, x, u);
  const double kx = floor(u[0]), ky = floor(u[1]), kz = floor(u[2]);
  x[0] = x[0] - ((kx * c->L[0] + ky * c->T[0]) + kz * c->T[1]);
  x[1] = x[1] - (ky * c->L[1] + kz * c->T[2]);
  x[2] = x[2] - kz * c->L[2];
}

/* widths of the cell between opposite faces */
static void cell_widths(const ro_ctx *c, double *w) {
  const double lx = c->L[0], ly = c->L[1], lz = c->L[2];
  const double xy = c->T[0], xz = c->T[1], yz = c->T[2];
  w[0] = lx; w[1] = ly; w[2] = lz;
  if (c->tri) {
    const double V = lx * ly * lz;
    w[0] = V / sqrt(ly * lz * ly * lz + xy * lz * xy * lz + (xy * yz - ly * xz) * (xy * yz - ly * xz));
    w[1] = ly * lz / sqrt(lz * lz + yz * yz);
  }
}

void ro_set_tilt(ro_ctx *c, const double *tilt3) {
  int d;
  for (d = 0; d < 3; d++) c->T[d] = tilt3 ? tilt3[d] : 0.0;
  c->tri = c->T[0] != 0.0 || c->T[1] != 0.0 || c->T[2] != 0.0;
}

int ro_set_system(ro_ctx *c, int n, const double *box3, const double *x,
                  const int *type, const int *tag, const double *q,
                  const double *v) {
  int i, d;
  if (n != c->n) {
    free(c->x); free(c->v); free(c->q); free(c->f); free(c->type);
    free(c->tag); free(c->s_hist); free(c->t_hist); free(c->s); free(c->t);
    free(c->cd_local);
    c->x = (double *)calloc(3 * (size_t)n, sizeof(double));
    c->v = (double *)calloc(3 * (size_t)n, sizeof(double));
    c->f = (double *)calloc(3 * (size_t)n, sizeof(double));
    c->q = (double *)calloc((size_t)n, sizeof(double));
    c->type = (int *)calloc((size_t)n, sizeof(int));
    c->tag = (int *)calloc((size_t)n, sizeof(int));
    c->s_hist = (double *)calloc(5 * (size_t)n, sizeof(double));
    c->t_hist = (double *)calloc(5 * (size_t)n, sizeof(double));
    c->s = (double *)calloc((size_t)n, sizeof(double));
    c->t = (double *)calloc((size_t)n, sizeof(double));
    c->cd_local = (double *)calloc((size_t)n, sizeof(double));
    c->n = n;
  } else {
    memset(c->s_hist, 0, 5 * (size_t)n * sizeof(double));
    memset(c->t_hist, 0, 5 * (size_t)n * sizeof(double));
  }
  for (d = 0; d < 3; d++) c->L[d] = box3[d];
  for (i = 0; i < n; i++) {
    if (type[i] < 0 || type[i] >= c->ff.ntypes) return -1;
    for (d = 0; d < 3; d++) c->x[3 * i + d] = x[3 * i + d];
    wrap_pos(c, c->x + 3 * i);
    c->type[i] = type[i];
    c->tag[i] = tag ? tag[i] : i + 1;
    c->q[i] = q ? q[i] : 0.0;
    for (d = 0; d < 3; d++) c->v[3 * i + d] = v ? v[3 * i + d] : 0.0;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* ghosts + binned full far-neighbour list
 * LAMMPS ghost atoms (Comm, absent) restated as periodic images within
 * cutghost of the box; full neighbour list npair_full_bin_ghost_sw5.c:80-231
 * filtered to d <= nonb_cut as write_reax_lists_c, pair_reaxc_sw64.c:42-96
 * (CPU form pair_reaxc_sunway.cpp:913-935). */

static int img_code(int sx, int sy, int sz) {
  return (sx + 8) | ((sy + 8) << 4) | ((sz + 8) << 8);
}

static void *xrealloc(void *p, size_t sz) {
  void *q = realloc(p, sz);
  if (!q && sz) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return q;
}

static void ensure_N(ro_ctx *c, int N) {
  if (N <= c->capN) return;
  int cap = N + N / 4 + 16;
#define GROWD(p, k) c->p = (double *)xrealloc(c->p, (size_t)cap * (k) * sizeof(double))
#define GROWI(p, k) c->p = (int *)xrealloc(c->p, (size_t)cap * (k) * sizeof(int))
  GROWD(xe, 3); GROWI(te, 1); GROWI(own, 1); GROWI(imgc, 1);
  GROWI(far_start, 1); c->far_start = (int *)xrealloc(c->far_start, ((size_t)cap + 1) * sizeof(int));
  GROWI(b_start, 1); GROWI(b_end, 1);
  GROWD(bo_dboc0, 1); GROWD(bo_dboc1, 1); GROWD(Deltap, 1); GROWD(Deltap_boc, 1);
  GROWD(Delta, 1); GROWD(Delta_e, 1); GROWD(Delta_val, 1); GROWD(vlpex, 1);
  GROWD(nlp, 1); GROWD(nlp_temp, 1); GROWD(Delta_lp, 1); GROWD(Delta_lp_temp, 1);
  GROWD(dDelta_lp, 1); GROWD(dDelta_lp_temp, 1); GROWD(Clp, 1);
  GROWD(dDeltap_self, 3); GROWD(fC, 4);
#undef GROWD
#undef GROWI
  c->capN = cap;
}

static void build_ghosts(ro_ctx *c) {
  const double cutmax =
      fmax(fmax(c->nonb_cut, c->ctl.hbond_cut), 2.0 * c->ctl.bond_cut);
  const double rc = cutmax + c->ctl.skin;
  int kmax[3], d, i, sx, sy, sz, N;
  double w[3];
  cell_widths(c, w);
  for (d = 0; d < 3; d++) kmax[d] = (int)ceil(rc / w[d]);
  ensure_N(c, c->n);
  for (i = 0; i < c->n; i++) {
    for (d = 0; d < 3; d++) c->xe[3 * i + d] = c->x[3 * i + d];
    c->te[i] = c->type[i];
    c->own[i] = i;
    c->imgc[i] = img_code(0, 0, 0);
  }
  N = c->n;
  for (sz = -kmax[2]; sz <= kmax[2]; sz++)
    for (sy = -kmax[1]; sy <= kmax[1]; sy++)
      for (sx = -kmax[0]; sx <= kmax[0]; sx++) {
        if (!sx && !sy && !sz) continue;
        double iv[3];
        const int s3[3] = {sx, sy, sz};
        img_vec(c, sx, sy, sz, iv);
        for (i = 0; i < c->n; i++) {
          double p[3];
          int ok = 1;
          if (!c->tri) {
            p[0] = c->x[3 * i + 0] + sx * c->L[0];
            p[1] = c->x[3 * i + 1] + sy * c->L[1];
            p[2] = c->x[3 * i + 2] + sz * c->L[2];
            for (d = 0; d < 3; d++)
              if (p[d] < -rc || p[d] >= c->L[d] + rc) ok = 0;
          } else {
            /* within rc of the cell across each pair of faces */
            double u[3];
            frac3(c, c->x + 3 * i, u);
            for (d = 0; d < 3; d++) {
              p[d] = c->x[3 * i + d] + iv[d];
              if (u[d] + s3[d] < -rc / w[d] || u[d] + s3[d] >= 1.0 + rc / w[d]) ok = 0;
            }
          }
          if (!ok) continue;
          ensure_N(c, N + 1);
          for (d = 0; d < 3; d++) c->xe[3 * N + d] = p[d];
          c->te[N] = c->type[i];
          c->own[N] = i;
          c->imgc[N] = img_code(sx, sy, sz);
          N++;
        }
      }
  c->N = N;
}

static void build_far(ro_ctx *c) {
  const double cut = c->nonb_cut;
  const double cutsq = cut * cut;
  double lo[3], hi[3];
  int nb[3], d, i, N = c->N;
  for (d = 0; d < 3; d++) {
    lo[d] = c->xe[d];
    hi[d] = c->xe[d];
  }
  for (i = 0; i < N; i++)
    for (d = 0; d < 3; d++) {
      if (c->xe[3 * i + d] < lo[d]) lo[d] = c->xe[3 * i + d];
      if (c->xe[3 * i + d] > hi[d]) hi[d] = c->xe[3 * i + d];
    }
  for (d = 0; d < 3; d++) {
    nb[d] = (int)((hi[d] - lo[d]) / cut);
    if (nb[d] < 1) nb[d] = 1;
  }
  long long nbins = (long long)nb[0] * nb[1] * nb[2];
  int *bin_head = (int *)malloc(nbins * sizeof(int));
  int *bin_next = (int *)malloc((size_t)N * sizeof(int));
  int *abin = (int *)malloc((size_t)N * 3 * sizeof(int));
  for (long long b = 0; b < nbins; b++) bin_head[b] = -1;
  for (i = N - 1; i >= 0; i--) {
    int bi[3];
    for (d = 0; d < 3; d++) {
      bi[d] = (int)((c->xe[3 * i + d] - lo[d]) / (hi[d] - lo[d] + 1e-12) * nb[d]);
      if (bi[d] >= nb[d]) bi[d] = nb[d] - 1;
      if (bi[d] < 0) bi[d] = 0;
      abin[3 * i + d] = bi[d];
    }
    long long b = ((long long)bi[2] * nb[1] + bi[1]) * nb[0] + bi[0];
    bin_next[i] = bin_head[b];
    bin_head[b] = i;
  }
  /* bin width >= cut so a 27-bin stencil suffices */
  long long top = 0;
  if (!c->far_cap) {
    c->far_cap = (long long)N * 64 + 1024;
    c->far_nbr = (int *)xrealloc(c->far_nbr, c->far_cap * sizeof(int));
    c->far_d = (double *)xrealloc(c->far_d, c->far_cap * sizeof(double));
    c->far_dvec = (double *)xrealloc(c->far_dvec, c->far_cap * 3 * sizeof(double));
  }
  for (i = 0; i < N; i++) {
    c->far_start[i] = (int)top;
    int bx, by, bz;
    for (bz = abin[3 * i + 2] - 1; bz <= abin[3 * i + 2] + 1; bz++) {
      if (bz < 0 || bz >= nb[2]) continue;
      for (by = abin[3 * i + 1] - 1; by <= abin[3 * i + 1] + 1; by++) {
        if (by < 0 || by >= nb[1]) continue;
        for (bx = abin[3 * i] - 1; bx <= abin[3 * i] + 1; bx++) {
          if (bx < 0 || bx >= nb[0]) continue;
          long long b = ((long long)bz * nb[1] + by) * nb[0] + bx;
          int j;
          for (j = bin_head[b]; j >= 0; j = bin_next[j]) {
            if (j == i) continue;
            double dv[3], dsq;
            dv[0] = c->xe[3 * j + 0] - c->xe[3 * i + 0];
            dv[1] = c->xe[3 * j + 1] - c->xe[3 * i + 1];
            dv[2] = c->xe[3 * j + 2] - c->xe[3 * i + 2];
            dsq = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
            if (dsq <= cutsq) {
              if (top >= c->far_cap) {
                c->far_cap = c->far_cap * 2;
                c->far_nbr = (int *)xrealloc(c->far_nbr, c->far_cap * sizeof(int));
                c->far_d = (double *)xrealloc(c->far_d, c->far_cap * sizeof(double));
                c->far_dvec = (double *)xrealloc(c->far_dvec, c->far_cap * 3 * sizeof(double));
              }
              c->far_nbr[top] = j;
              c->far_d[top] = sqrt(dsq);
              c->far_dvec[3 * top + 0] = dv[0];
              c->far_dvec[3 * top + 1] = dv[1];
              c->far_dvec[3 * top + 2] = dv[2];
              top++;
            }
          }
        }
      }
    }
  }
  c->far_start[N] = (int)top;
  free(bin_head);
  free(bin_next);
  free(abin);
}

/* ------------------------------------------------------------------ */
/* uncorrected bond orders + full bond list: BOp_single and
 * Init_Forces_noQEq_Full, reaxc_forces_sunway.cpp:677-934 (libm form of
 * Init_Forces_noQEq_Full_C_para reaxc_forces_sw64.c:996-1318, including
 * the per-atom sort by neighbour index :1284-1291 / my_bubble_sort :31) */

static void build_bonds(ro_ctx *c) {
  int i, N = c->N;
  long long top = 0, far_tot = c->far_start[N];
  if (c->bond_cap < far_tot / 4 + 1024) {
    c->bond_cap = far_tot / 4 + 1024;
    c->bonds = (bond_t *)xrealloc(c->bonds, c->bond_cap * sizeof(bond_t));
  }
  for (i = 0; i < N; i++) {
    c->bo_dboc0[i] = 0.0;
    c->dDeltap_self[3 * i] = c->dDeltap_self[3 * i + 1] = c->dDeltap_self[3 * i + 2] = 0.0;
  }
  for (i = 0; i < N; i++) {
    int ti = c->te[i];
    const sbp_t *sbp_i = &c->ff.sbp[ti];
    int pj;
    c->b_start[i] = (int)top;
    for (pj = c->far_start[i]; pj < c->far_start[i + 1]; pj++) {
      double d = c->far_d[pj];
      if (!(d <= c->ctl.bond_cut)) continue;
      int j = c->far_nbr[pj], tj = c->te[j];
      const sbp_t *sbp_j = &c->ff.sbp[tj];
      const tbp_t *tw = &c->ff.tbp[ti][tj];
      double C12, C34, C56, BO_s, BO_pi, BO_pi2, BO;
      double r2 = SQR(d);
      if (sbp_i->r_s > 0.0 && sbp_j->r_s > 0.0) {
        C12 = tw->p_bo1 * pow(d / tw->r_s, tw->p_bo2);
        BO_s = (1.0 + c->bo_cut) * exp(C12);
      } else BO_s = C12 = 0.0;
      if (sbp_i->r_pi > 0.0 && sbp_j->r_pi > 0.0) {
        C34 = tw->p_bo3 * pow(d / tw->r_p, tw->p_bo4);
        BO_pi = exp(C34);
      } else BO_pi = C34 = 0.0;
      if (sbp_i->r_pi_pi > 0.0 && sbp_j->r_pi_pi > 0.0) {
        C56 = tw->p_bo5 * pow(d / tw->r_pp, tw->p_bo6);
        BO_pi2 = exp(C56);
      } else BO_pi2 = C56 = 0.0;
      BO = BO_s + BO_pi + BO_pi2;
      if (BO >= c->bo_cut) {
        if (top >= c->bond_cap) {
          c->bond_cap *= 2;
          c->bonds = (bond_t *)xrealloc(c->bonds, c->bond_cap * sizeof(bond_t));
        }
        bond_t *b = &c->bonds[top];
        memset(b, 0, sizeof *b);
        int k;
        b->nbr = j;
        b->far = pj;
        b->d = d;
        for (k = 0; k < 3; k++) b->dvec[k] = c->far_dvec[3 * pj + k];
        b->BO = BO;
        b->BO_s = BO_s;
        b->BO_pi = BO_pi;
        b->BO_pi2 = BO_pi2;
        double Cln_BOp_s = tw->p_bo2 * C12 / r2;
        double Cln_BOp_pi = tw->p_bo4 * C34 / r2;
        double Cln_BOp_pi2 = tw->p_bo6 * C56 / r2;
        for (k = 0; k < 3; k++) {
          b->dln_BOp_s[k] = -b->BO_s * Cln_BOp_s * b->dvec[k];
          b->dln_BOp_pi[k] = -b->BO_pi * Cln_BOp_pi * b->dvec[k];
          b->dln_BOp_pi2[k] = -b->BO_pi2 * Cln_BOp_pi2 * b->dvec[k];
          b->dBOp[k] = -(b->BO_s * Cln_BOp_s + b->BO_pi * Cln_BOp_pi +
                         b->BO_pi2 * Cln_BOp_pi2) * b->dvec[k];
          c->dDeltap_self[3 * i + k] += b->dBOp[k];
        }
        b->BO_s -= c->bo_cut;
        b->BO -= c->bo_cut;
        c->bo_dboc0[i] += b->BO;
        top++;
      }
    }
    c->b_end[i] = (int)top;
    /* stable sort of i's bonds by neighbour index */
    {
      int s = c->b_start[i], e = c->b_end[i], a;
      for (a = s + 1; a < e; a++) {
        bond_t tmp = c->bonds[a];
        int z = a - 1;
        while (z >= s && c->bonds[z].nbr > tmp.nbr) {
          c->bonds[z + 1] = c->bonds[z];
          z--;
        }
        c->bonds[z + 1] = tmp;
      }
    }
  }
  /* sym_index: BO_Section2_C CPU form, reaxc_bond_orders_sw64.c:182-195
   * (last match wins) */
  for (i = 0; i < N; i++) {
    int pj;
    for (pj = c->b_start[i]; pj < c->b_end[i]; pj++) {
      int j = c->bonds[pj].nbr, pk;
      c->bonds[pj].sym = -1;
      for (pk = c->b_start[j]; pk < c->b_end[j]; pk++)
        if (c->bonds[pk].nbr == i) c->bonds[pj].sym = pk;
    }
  }
}

/* H-bond list: Init_Forces_noQEq_HB_Full_C, reaxc_forces_sw64.c:787-863 */
static void build_hbonds(ro_ctx *c) {
  int i;
  long long top = 0;
  c->hb_start = (int *)xrealloc(c->hb_start, ((size_t)c->n + 1) * sizeof(int));
  if (!c->hb_cap) {
    c->hb_cap = 1024;
    c->hb_far = (int *)xrealloc(c->hb_far, c->hb_cap * sizeof(int));
  }
  for (i = 0; i < c->n; i++) {
    c->hb_start[i] = (int)top;
    if (c->ctl.hbond_cut <= 0) continue;
    if (c->ff.sbp[c->te[i]].p_hbond != 1) continue;
    int pj;
    for (pj = c->far_start[i]; pj < c->far_start[i + 1]; pj++) {
      if (!(c->far_d[pj] <= c->ctl.hbond_cut)) continue;
      int j = c->far_nbr[pj];
      if (c->ff.sbp[c->te[j]].p_hbond == 2) {
        if (top >= c->hb_cap) {
          c->hb_cap *= 2;
          c->hb_far = (int *)xrealloc(c->hb_far, c->hb_cap * sizeof(int));
        }
        c->hb_far[top++] = pj;
      }
    }
  }
  c->hb_start[c->n] = (int)top;
}

/* ------------------------------------------------------------------ */
/* bond-order correction: BO_Section1/2/3_C CPU forms,
 * reaxc_bond_orders_sw64.c:56-64, :162-377, :451-482 */

static void bond_orders(ro_ctx *c) {
  int i, N = c->N;
  const double p_boc1 = c->ff.gp[0], p_boc2 = c->ff.gp[1];
  const double p_lp1 = c->ff.gp[15];
  for (i = 0; i < N; i++) {
    const sbp_t *s = &c->ff.sbp[c->te[i]];
    c->Deltap[i] = c->bo_dboc0[i] - s->valency;
    c->Deltap_boc[i] = c->bo_dboc0[i] - s->valency_val;
    c->bo_dboc0[i] = 0;
  }
  for (i = 0; i < N; i++) {
    int ti = c->te[i], pj;
    double val_i = c->ff.sbp[ti].valency;
    double Deltap_i = c->Deltap[i], Deltap_boc_i = c->Deltap_boc[i];
    for (pj = c->b_start[i]; pj < c->b_end[i]; pj++) {
      bond_t *b = &c->bonds[pj];
      int j = b->nbr, tj = c->te[j];
      const tbp_t *tw = &c->ff.tbp[ti][tj];
      if (tw->ovc < 0.001 && tw->v13cor < 0.001) {
        b->C1dbo = 1.0; b->C2dbo = 0.0; b->C3dbo = 0.0;
        b->C1dbopi = b->BO_pi; b->C2dbopi = 0; b->C3dbopi = 0; b->C4dbopi = 0;
        b->C1dbopi2 = b->BO_pi2; b->C2dbopi2 = 0; b->C3dbopi2 = 0; b->C4dbopi2 = 0;
      } else {
        double val_j = c->ff.sbp[tj].valency;
        double Deltap_j = c->Deltap[j], Deltap_boc_j = c->Deltap_boc[j];
        double f1, Cf1_ij, Cf1_ji, f4, f5, f4f5, Cf45_ij, Cf45_ji;
        if (tw->ovc >= 0.001) {
          double exp_p1i = exp(-p_boc1 * Deltap_i);
          double exp_p2i = exp(-p_boc2 * Deltap_i);
          double exp_p1j = exp(-p_boc1 * Deltap_j);
          double exp_p2j = exp(-p_boc2 * Deltap_j);
          double f2 = exp_p1i + exp_p1j;
          double f3 = -1.0 / p_boc2 * log(0.5 * (exp_p2i + exp_p2j));
          f1 = 0.5 * ((val_i + f2) / (val_i + f2 + f3) +
                      (val_j + f2) / (val_j + f2 + f3));
          double temp = f2 + f3;
          double u1_ij = val_i + temp, u1_ji = val_j + temp;
          double Cf1A_ij = 0.5 * f3 * (1.0 / SQR(u1_ij) + 1.0 / SQR(u1_ji));
          double Cf1B_ij = -0.5 * ((u1_ij - f3) / SQR(u1_ij) +
                                   (u1_ji - f3) / SQR(u1_ji));
          Cf1_ij = 0.50 * (-p_boc1 * exp_p1i / u1_ij -
                           ((val_i + f2) / SQR(u1_ij)) *
                               (-p_boc1 * exp_p1i + exp_p2i / (exp_p2i + exp_p2j)) +
                           -p_boc1 * exp_p1i / u1_ji -
                           ((val_j + f2) / SQR(u1_ji)) *
                               (-p_boc1 * exp_p1i + exp_p2i / (exp_p2i + exp_p2j)));
          Cf1_ji = -Cf1A_ij * p_boc1 * exp_p1j +
                   Cf1B_ij * exp_p2j / (exp_p2i + exp_p2j);
        } else {
          f1 = 1.0;
          Cf1_ij = Cf1_ji = 0.0;
        }
        if (tw->v13cor >= 0.001) {
          double exp_f4 = exp(-(tw->p_boc4 * SQR(b->BO) - Deltap_boc_i) * tw->p_boc3 + tw->p_boc5);
          double exp_f5 = exp(-(tw->p_boc4 * SQR(b->BO) - Deltap_boc_j) * tw->p_boc3 + tw->p_boc5);
          f4 = 1. / (1. + exp_f4);
          f5 = 1. / (1. + exp_f5);
          f4f5 = f4 * f5;
          Cf45_ij = -f4 * exp_f4;
          Cf45_ji = -f5 * exp_f5;
        } else {
          f4 = f5 = f4f5 = 1.0;
          Cf45_ij = Cf45_ji = 0.0;
        }
        double A0_ij = f1 * f4f5;
        double A1_ij = -2 * tw->p_boc3 * tw->p_boc4 * b->BO * (Cf45_ij + Cf45_ji);
        double A2_ij = Cf1_ij / f1 + tw->p_boc3 * Cf45_ij;
        double A2_ji = Cf1_ji / f1 + tw->p_boc3 * Cf45_ji;
        double A3_ij = A2_ij + Cf1_ij / f1;
        double A3_ji = A2_ji + Cf1_ji / f1;
        b->BO = b->BO * A0_ij;
        b->BO_pi = b->BO_pi * A0_ij * f1;
        b->BO_pi2 = b->BO_pi2 * A0_ij * f1;
        b->BO_s = b->BO - (b->BO_pi + b->BO_pi2);
        b->C1dbo = A0_ij + b->BO * A1_ij;
        b->C2dbo = b->BO * A2_ij;
        b->C3dbo = b->BO * A2_ji;
        b->C1dbopi = f1 * f1 * f4 * f5;
        b->C2dbopi = b->BO_pi * A1_ij;
        b->C3dbopi = b->BO_pi * A3_ij;
        b->C4dbopi = b->BO_pi * A3_ji;
        b->C1dbopi2 = f1 * f1 * f4 * f5;
        b->C2dbopi2 = b->BO_pi2 * A1_ij;
        b->C3dbopi2 = b->BO_pi2 * A3_ij;
        b->C4dbopi2 = b->BO_pi2 * A3_ji;
      }
      if (b->BO < 1e-10) b->BO = 0.0;
      if (b->BO_s < 1e-10) b->BO_s = 0.0;
      if (b->BO_pi < 1e-10) b->BO_pi = 0.0;
      if (b->BO_pi2 < 1e-10) b->BO_pi2 = 0.0;
      c->bo_dboc0[i] += b->BO;
    }
  }
  for (i = 0; i < N; i++) {
    const sbp_t *s = &c->ff.sbp[c->te[i]];
    c->Delta[i] = c->bo_dboc0[i] - s->valency;
    c->Delta_e[i] = c->bo_dboc0[i] - s->valency_e;
    c->bo_dboc1[i] = c->bo_dboc0[i] - s->valency_boc;
    c->Delta_val[i] = c->bo_dboc0[i] - s->valency_val;
    c->vlpex[i] = c->Delta_e[i] - 2.0 * (int)(c->Delta_e[i] / 2.0);
    double explp1 = exp(-p_lp1 * SQR(2.0 + c->vlpex[i]));
    c->nlp[i] = explp1 - (int)(c->Delta_e[i] / 2.0);
    c->Delta_lp[i] = s->nlp_opt - c->nlp[i];
    c->Clp[i] = 2.0 * p_lp1 * explp1 * (2.0 + c->vlpex[i]);
    c->dDelta_lp[i] = c->Clp[i];
    if (s->mass > 21.0) {
      c->nlp_temp[i] = 0.5 * (s->valency_e - s->valency);
      c->Delta_lp_temp[i] = s->nlp_opt - c->nlp_temp[i];
      c->dDelta_lp_temp[i] = 0.;
    } else {
      c->nlp_temp[i] = c->nlp[i];
      c->Delta_lp_temp[i] = s->nlp_opt - c->nlp_temp[i];
      c->dDelta_lp_temp[i] = c->Clp[i];
    }
  }
}

/* tie-break used for bonds and torsions when both ends carry the same tag
 * (an atom bonded to its own image), reaxc_multi_body_sw64.c:256-267 */
static int tag_first(const ro_ctx *c, int i, int j) {
  int ti = c->tag[c->own[i]], tj = c->tag[c->own[j]];
  const double *xi = &c->xe[3 * i], *xj = &c->xe[3 * j];
  if (ti > tj) return 0;
  if (ti == tj) {
    if (xj[2] < xi[2]) return 0;
    if (xj[2] == xi[2] && xj[1] < xi[1]) return 0;
    if (xj[2] == xi[2] && xj[1] == xi[1] && xj[0] < xi[0]) return 0;
  }
  return 1;
}

/* ------------------------------------------------------------------ */
/* bond energy + lone pair + over/under-coordination + polarisation:
 * Merge_Bonds_Atom_Energy_C_New, reaxc_multi_body_sw64.c:21-333 */

static void atom_energy(ro_ctx *c) {
  const ffield_t *ff = &c->ff;
  const double p_lp3 = ff->gp[5], p_ovun3 = ff->gp[32], p_ovun4 = ff->gp[31];
  const double p_ovun6 = ff->gp[6], p_ovun7 = ff->gp[8], p_ovun8 = ff->gp[9];
  const double gp3 = ff->gp[3], gp4 = ff->gp[4], gp7 = ff->gp[7];
  const double gp10 = ff->gp[10];
  const int gp37 = (int)ff->gp[37];
  double e_lph = 0, e_lp = 0, e_ov = 0, ebond = 0, estriph = 0, e_un_sum = 0;
  double en_tmp = 0, e_pol = 0, e_pol_phys = 0;
  int i;
  for (i = 0; i < c->n; i++) {
    int ti = c->te[i], pj, numbonds = 0;
    const sbp_t *sbp_i = &ff->sbp[ti];
    double q = c->q[i];
    double pol = KCALpMOL_to_EV * (sbp_i->chi * q + (sbp_i->eta / 2.) * SQR(q));
    en_tmp += pol;
    e_pol += en_tmp; /* prefix-sum artefact of the reference (:102-103) */
    e_pol_phys += pol;
    double p_lp2 = sbp_i->p_lp2;
    double expvd2 = exp(-75 * c->Delta_lp[i]);
    double inv_expvd2 = 1. / (1. + expvd2);
    double p_ovun2 = sbp_i->p_ovun2;
    double sum_ovun1 = 0, sum_ovun2 = 0;
    double dfvl = (sbp_i->mass > 21.0) ? 0.0 : 1.0;
    for (pj = c->b_start[i]; pj < c->b_end[i]; pj++) {
      const bond_t *b = &c->bonds[pj];
      int j = b->nbr, tj = c->te[j];
      numbonds++;
      const tbp_t *tw = &ff->tbp[ti][tj];
      sum_ovun1 += tw->p_ovun1 * tw->De_s * b->BO;
      sum_ovun2 += (c->Delta[j] - dfvl * c->Delta_lp_temp[j]) * (b->BO_pi + b->BO_pi2);
    }
    double dElp = p_lp2 * inv_expvd2 +
                  75 * p_lp2 * c->Delta_lp[i] * expvd2 * SQR(inv_expvd2);
    double CElp = dElp * c->dDelta_lp[i];
    if (p_lp3 > 0.001 && !strcmp(sbp_i->name, "C")) {
      for (pj = c->b_start[i]; pj < c->b_end[i]; pj++) {
        bond_t *b = &c->bonds[pj];
        int j = b->nbr;
        if (!strcmp(ff->sbp[c->te[j]].name, "C")) {
          double Di = c->Delta[i];
          double vov3 = b->BO - Di - 0.040 * pow(Di, 4.);
          if (vov3 > 3.) {
            e_lph += p_lp3 * SQR(vov3 - 3.0);
            double deahu2dbo = 2. * p_lp3 * (vov3 - 3.);
            double deahu2dsbo = 2. * p_lp3 * (vov3 - 3.) * (-1. - 0.16 * pow(Di, 3.));
            b->Cdbo += deahu2dbo;
            c->fC[4 * i + 3] += deahu2dsbo;
          }
        }
      }
    }
    double exp_ovun1 = p_ovun3 * exp(p_ovun4 * sum_ovun2);
    double inv_exp_ovun1 = 1.0 / (1 + exp_ovun1);
    double Delta_lpcorr = c->Delta[i] - (dfvl * c->Delta_lp_temp[i]) * inv_exp_ovun1;
    double exp_ovun2 = exp(p_ovun2 * Delta_lpcorr);
    double inv_exp_ovun2 = 1.0 / (1.0 + exp_ovun2);
    double DlpVi = 1.0 / (Delta_lpcorr + sbp_i->valency + 1e-8);
    double CEover1 = Delta_lpcorr * DlpVi * inv_exp_ovun2;
    e_ov += sum_ovun1 * CEover1;
    double CEover2 = sum_ovun1 * DlpVi * inv_exp_ovun2 *
                     (1.0 - Delta_lpcorr * (DlpVi + p_ovun2 * exp_ovun2 * inv_exp_ovun2));
    double CEover3 = CEover2 * (1.0 - dfvl * c->dDelta_lp[i] * inv_exp_ovun1);
    double CEover4 = CEover2 * (dfvl * c->Delta_lp_temp[i]) * p_ovun4 *
                     exp_ovun1 * SQR(inv_exp_ovun1);
    double p_ovun5 = sbp_i->p_ovun5;
    double exp_ovun2n = 1.0 / exp_ovun2;
    double exp_ovun6 = exp(p_ovun6 * Delta_lpcorr);
    double exp_ovun8 = p_ovun7 * exp(p_ovun8 * sum_ovun2);
    double inv_exp_ovun2n = 1.0 / (1.0 + exp_ovun2n);
    double inv_exp_ovun8 = 1.0 / (1.0 + exp_ovun8);
    double e_un = 0.0, CEunder1, CEunder2, CEunder3, CEunder4;
    c->fC[4 * i + 3] += CEover3;
    if (numbonds > 0 || c->ctl.enobondsflag) {
      e_un = -p_ovun5 * (1.0 - exp_ovun6) * inv_exp_ovun2n * inv_exp_ovun8;
      e_un_sum += e_un;
      CEunder1 = inv_exp_ovun2n * (p_ovun5 * p_ovun6 * exp_ovun6 * inv_exp_ovun8 +
                                   p_ovun2 * e_un * exp_ovun2n);
      CEunder2 = -e_un * p_ovun8 * exp_ovun8 * inv_exp_ovun8;
      CEunder3 = CEunder1 * (1.0 - dfvl * c->dDelta_lp[i] * inv_exp_ovun1);
      CEunder4 = CEunder1 * (dfvl * c->Delta_lp_temp[i]) * p_ovun4 * exp_ovun1 *
                     SQR(inv_exp_ovun1) + CEunder2;
      c->fC[4 * i + 3] += CEunder3;
      c->fC[4 * i + 3] += CElp;
      e_lp += p_lp2 * c->Delta_lp[i] * inv_expvd2;
    } else {
      CEunder1 = inv_exp_ovun2n * (p_ovun5 * p_ovun6 * exp_ovun6 * inv_exp_ovun8 +
                                   p_ovun2 * e_un * exp_ovun2n);
      CEunder2 = -e_un * p_ovun8 * exp_ovun8 * inv_exp_ovun8;
      CEunder3 = CEunder1 * (1.0 - dfvl * c->dDelta_lp[i] * inv_exp_ovun1);
      CEunder4 = CEunder1 * (dfvl * c->Delta_lp_temp[i]) * p_ovun4 * exp_ovun1 *
                     SQR(inv_exp_ovun1) + CEunder2;
    }
    for (pj = c->b_start[i]; pj < c->b_end[i]; pj++) {
      bond_t *b = &c->bonds[pj];
      int j = b->nbr, tj = c->te[j];
      const tbp_t *tw = &ff->tbp[ti][tj];
      b->Cdbo += CEover1 * tw->p_ovun1 * tw->De_s;
      double ftmp2 = (1.0 - dfvl * c->dDelta_lp[j]) * (b->BO_pi + b->BO_pi2);
      c->fC[4 * j + 3] += CEover4 * ftmp2;
      double ftmp = CEover4 * (c->Delta[j] - dfvl * c->Delta_lp_temp[j]);
      b->Cdbopi += ftmp;
      b->Cdbopi2 += ftmp;
      c->fC[4 * j + 3] += CEunder4 * ftmp2;
      double fc3 = CEunder4 * (c->Delta[j] - dfvl * c->Delta_lp_temp[j]);
      b->Cdbopi += fc3;
      b->Cdbopi2 += fc3;
      if (tag_first(c, i, j)) {
        const sbp_t *sbp_j = &ff->sbp[tj];
        double pow_BOs_be2 = (b->BO_s == 0.0) ? 0.0 : pow(b->BO_s, tw->p_be2);
        double exp_be12 = exp(tw->p_be1 * (1.0 - pow_BOs_be2));
        double CEbo = -tw->De_s * exp_be12 * (1.0 - tw->p_be1 * tw->p_be2 * pow_BOs_be2);
        ebond += -tw->De_s * b->BO_s * exp_be12 - tw->De_p * b->BO_pi -
                 tw->De_pp * b->BO_pi2;
        b->Cdbo += CEbo;
        b->Cdbopi -= (CEbo + tw->De_p);
        b->Cdbopi2 -= (CEbo + tw->De_pp);
        if (b->BO >= 1.00) {
          if (gp37 == 2 || (sbp_i->mass == 12.0000 && sbp_j->mass == 15.9990) ||
              (sbp_j->mass == 12.0000 && sbp_i->mass == 15.9990)) {
            double exphu = exp(-gp7 * SQR(b->BO - 2.50));
            double exphua1 = exp(-gp3 * (c->bo_dboc0[i] - b->BO));
            double exphub1 = exp(-gp3 * (c->bo_dboc0[j] - b->BO));
            double exphuov = exp(gp4 * (c->Delta[i] + c->Delta[j]));
            double hulpov = 1.0 / (1.0 + 25.0 * exphuov);
            estriph += gp10 * exphu * hulpov * (exphua1 + exphub1);
            double decobdbo = gp10 * exphu * hulpov * (exphua1 + exphub1) *
                              (gp3 - 2.0 * gp7 * (b->BO - 2.50));
            double decobdboua = -gp10 * exphu * hulpov *
                                (gp3 * exphua1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1));
            double decobdboub = -gp10 * exphu * hulpov *
                                (gp3 * exphub1 + 25.0 * gp4 * exphuov * hulpov * (exphua1 + exphub1));
            b->Cdbo += decobdbo;
            c->fC[4 * i + 3] += decobdboua;
            c->fC[4 * j + 3] += decobdboub;
          }
        }
      }
    }
  }
  c->en[RO_ENG_VDWL] += e_un_sum + (e_lph + e_lp + e_ov + ebond + estriph);
  c->en[RO_ENG_COUL] += en_tmp;
  c->en[RO_E_POL] = e_pol;
  c->en[RO_E_POL_PHYS] = e_pol_phys;
  c->en[RO_E_LP] += e_lph + e_lp;
  c->en[RO_E_OVUN] += e_ov + e_un_sum;
  c->en[RO_E_BOND] += ebond + estriph;
}

/* Calculate_Theta / Calculate_dCos_Theta,
 * reaxc_valence_angles_sunway.cpp:49-79 */
static void calc_theta(const double *dji, double d_ji, const double *djk,
                       double d_jk, double *theta, double *cos_theta) {
  double dot = dji[0] * djk[0] + dji[1] * djk[1] + dji[2] * djk[2];
  *cos_theta = dot / (d_ji * d_jk);
  if (*cos_theta > 1.) *cos_theta = 1.0;
  if (*cos_theta < -1.) *cos_theta = -1.0;
  *theta = acos(*cos_theta);
}

static void calc_dcos_theta(const double *dji, double d_ji, const double *djk,
                            double d_jk, double *di, double *dj, double *dk) {
  double sqr_d_ji = SQR(d_ji), sqr_d_jk = SQR(d_jk);
  double inv_dists = 1.0 / (d_ji * d_jk);
  double inv_dists3 = pow(inv_dists, 3.0);
  double dot = dji[0] * djk[0] + dji[1] * djk[1] + dji[2] * djk[2];
  double Cdot_inv3 = dot * inv_dists3;
  int t;
  for (t = 0; t < 3; t++) {
    di[t] = djk[t] * inv_dists - Cdot_inv3 * sqr_d_jk * dji[t];
    dj[t] = -(djk[t] + dji[t]) * inv_dists +
            Cdot_inv3 * (sqr_d_jk * dji[t] + sqr_d_ji * djk[t]);
    dk[t] = dji[t] * inv_dists - Cdot_inv3 * sqr_d_ji * djk[t];
  }
}

static void add4(double *fc, double s, const double *v) {
  fc[0] += s * v[0];
  fc[1] += s * v[1];
  fc[2] += s * v[2];
}

/* ------------------------------------------------------------------ */
/* hydrogen bonds: Hydrogen_Bonds_C CPU form,
 * reaxc_hydrogen_bonds_sw64.c:146-248 */

static void hydrogen_bonds(ro_ctx *c) {
  const ffield_t *ff = &c->ff;
  double e_hb_sum = 0;
  int j;
  int hblist[256];
  for (j = 0; j < c->n; j++) {
    int tj = c->te[j];
    if (ff->sbp[tj].p_hbond != 1) continue;
    int top = 0, pi, pk, itr;
    for (pi = c->b_start[j]; pi < c->b_end[j]; pi++) {
      int i = c->bonds[pi].nbr;
      if (ff->sbp[c->te[i]].p_hbond == 2 && c->bonds[pi].BO >= HB_THRESHOLD && top < 256)
        hblist[top++] = pi;
    }
    for (pk = c->hb_start[j]; pk < c->hb_start[j + 1]; pk++) {
      int fk = c->hb_far[pk];
      int k = c->far_nbr[fk], tk = c->te[k];
      double r_jk = c->far_d[fk];
      const double *dvec_jk = &c->far_dvec[3 * fk];
      for (itr = 0; itr < top; itr++) {
        pi = hblist[itr];
        bond_t *b = &c->bonds[pi];
        int i = b->nbr;
        if (c->tag[c->own[i]] == c->tag[c->own[k]]) continue;
        int ti = c->te[i];
        const hbp_t *hbp = &ff->hbp[ti][tj][tk];
        if (hbp->r0_hb <= 0.0) continue;
        double theta, cos_theta, di[3], dj[3], dk[3];
        calc_theta(b->dvec, b->d, dvec_jk, r_jk, &theta, &cos_theta);
        calc_dcos_theta(b->dvec, b->d, dvec_jk, r_jk, di, dj, dk);
        double sin_theta2 = sin(theta / 2.0);
        double sin_xhz4 = SQR(sin_theta2);
        sin_xhz4 *= sin_xhz4;
        double cos_xhz1 = (1.0 - cos_theta);
        double exp_hb2 = exp(-hbp->p_hb2 * b->BO);
        double exp_hb3 = exp(-hbp->p_hb3 * (hbp->r0_hb / r_jk + r_jk / hbp->r0_hb - 2.0));
        double e_hb = hbp->p_hb1 * (1.0 - exp_hb2) * exp_hb3 * sin_xhz4;
        e_hb_sum += e_hb;
        double CEhb1 = hbp->p_hb1 * hbp->p_hb2 * exp_hb2 * exp_hb3 * sin_xhz4;
        double CEhb2 = -hbp->p_hb1 / 2.0 * (1.0 - exp_hb2) * exp_hb3 * cos_xhz1;
        double CEhb3 = -hbp->p_hb3 * (-hbp->r0_hb / SQR(r_jk) + 1.0 / hbp->r0_hb) * e_hb;
        b->Cdbo += CEhb1;
        add4(&c->fC[4 * i], +CEhb2, di);
        add4(&c->fC[4 * j], +CEhb2, dj);
        add4(&c->fC[4 * k], +CEhb2, dk);
        add4(&c->fC[4 * j], -CEhb3 / r_jk, dvec_jk);
        add4(&c->fC[4 * k], +CEhb3 / r_jk, dvec_jk);
      }
    }
  }
  c->en[RO_E_HB] += e_hb_sum;
  c->en[RO_ENG_VDWL] += e_hb_sum;
}

/* ------------------------------------------------------------------ */
/* Calculate_Omega, reaxc_torsion_angles_sw64.c:21-102 */
typedef struct {
  double theta, dcos_di[3], dcos_dj[3], dcos_dk[3];
} thb_t;

static double calc_omega(const double *dvec_ij, double r_ij,
                         const double *dvec_jk, double r_jk,
                         const double *dvec_kl, double r_kl,
                         const double *dvec_li, double r_li, const thb_t *p_ijk,
                         const thb_t *p_jkl, double *dcos_omega_di,
                         double *dcos_omega_dj, double *dcos_omega_dk,
                         double *dcos_omega_dl) {
  double sin_ijk = sin(p_ijk->theta), cos_ijk = cos(p_ijk->theta);
  double sin_jkl = sin(p_jkl->theta), cos_jkl = cos(p_jkl->theta);
  double dij_jk = dvec_ij[0] * dvec_jk[0] + dvec_ij[1] * dvec_jk[1] + dvec_ij[2] * dvec_jk[2];
  double djk_kl = dvec_jk[0] * dvec_kl[0] + dvec_jk[1] * dvec_kl[1] + dvec_jk[2] * dvec_kl[2];
  double dij_kl = dvec_ij[0] * dvec_kl[0] + dvec_ij[1] * dvec_kl[1] + dvec_ij[2] * dvec_kl[2];
  double unnorm_cos_omega = -dij_jk * djk_kl + SQR(r_jk) * dij_kl;
  double cr[3];
  cr[0] = dvec_jk[1] * dvec_kl[2] - dvec_jk[2] * dvec_kl[1];
  cr[1] = dvec_jk[2] * dvec_kl[0] - dvec_jk[0] * dvec_kl[2];
  cr[2] = dvec_jk[0] * dvec_kl[1] - dvec_jk[1] * dvec_kl[0];
  double unnorm_sin_omega =
      -r_jk * (dvec_ij[0] * cr[0] + dvec_ij[1] * cr[1] + dvec_ij[2] * cr[2]);
  double omega = atan2(unnorm_sin_omega, unnorm_cos_omega);
  double htra = r_ij + cos_ijk * (r_kl * cos_jkl - r_jk);
  double htrb = r_jk - r_ij * cos_ijk - r_kl * cos_jkl;
  double htrc = r_kl + cos_jkl * (r_ij * cos_ijk - r_jk);
  double hthd = r_ij * sin_ijk * (r_jk - r_kl * cos_jkl);
  double hthe = r_kl * sin_jkl * (r_jk - r_ij * cos_ijk);
  double hnra = r_kl * sin_ijk * sin_jkl;
  double hnrc = r_ij * sin_ijk * sin_jkl;
  double hnhd = r_ij * r_kl * cos_ijk * sin_jkl;
  double hnhe = r_ij * r_kl * sin_ijk * cos_jkl;
  double poem = 2.0 * r_ij * r_kl * sin_ijk * sin_jkl;
  if (poem < 1e-20) poem = 1e-20;
  double tel = SQR(r_ij) + SQR(r_jk) + SQR(r_kl) - SQR(r_li) -
               2.0 * (r_ij * r_jk * cos_ijk - r_ij * r_kl * cos_ijk * cos_jkl +
                      r_jk * r_kl * cos_jkl);
  double arg = tel / poem;
  if (arg > 1.0) arg = 1.0;
  if (arg < -1.0) arg = -1.0;
  if (sin_ijk >= 0 && sin_ijk <= MIN_SINE) sin_ijk = MIN_SINE;
  else if (sin_ijk <= 0 && sin_ijk >= -MIN_SINE) sin_ijk = -MIN_SINE;
  if (sin_jkl >= 0 && sin_jkl <= MIN_SINE) sin_jkl = MIN_SINE;
  else if (sin_jkl <= 0 && sin_jkl >= -MIN_SINE) sin_jkl = -MIN_SINE;
  int t;
  double a;
  for (t = 0; t < 3; t++) {
    a = (htra - arg * hnra) / r_ij * dvec_ij[t] - dvec_li[t];
    a += -(hthd - arg * hnhd) / sin_ijk * p_ijk->dcos_dk[t];
    dcos_omega_di[t] = 2.0 / poem * a;
    a = -(htra - arg * hnra) / r_ij * dvec_ij[t] - htrb / r_jk * dvec_jk[t];
    a += -(hthd - arg * hnhd) / sin_ijk * p_ijk->dcos_dj[t];
    a += -(hthe - arg * hnhe) / sin_jkl * p_jkl->dcos_di[t];
    dcos_omega_dj[t] = 2.0 / poem * a;
    a = -(htrc - arg * hnrc) / r_kl * dvec_kl[t] + htrb / r_jk * dvec_jk[t];
    a += -(hthd - arg * hnhd) / sin_ijk * p_ijk->dcos_di[t];
    a += -(hthe - arg * hnhe) / sin_jkl * p_jkl->dcos_dj[t];
    dcos_omega_dk[t] = 2.0 / poem * a;
    a = (htrc - arg * hnrc) / r_kl * dvec_kl[t] + dvec_li[t];
    a += -(hthe - arg * hnhe) / sin_jkl * p_jkl->dcos_dk[t];
    dcos_omega_dl[t] = 2.0 / poem * a;
  }
  return omega;
}

/* ------------------------------------------------------------------ */
/* valence + penalty + coalition + torsion + conjugation, merged:
 * Merge_Torsion_Valence_Angles CPU form, reaxc_torsion_angles_sw64.c:813-1367 */

static void torsion_valence(ro_ctx *c) {
  const ffield_t *ff = &c->ff;
  const double p_tor2 = ff->gp[23], p_tor3 = ff->gp[24], p_tor4 = ff->gp[25];
  const double p_cot2 = ff->gp[27], p_val6 = ff->gp[14], p_val8 = ff->gp[33];
  const double p_val9 = ff->gp[16], p_val10 = ff->gp[17];
  const double p_pen2 = ff->gp[19], p_pen3 = ff->gp[20], p_pen4 = ff->gp[21];
  const double p_coa2 = ff->gp[2], p_coa3 = ff->gp[38], p_coa4 = ff->gp[30];
  const double thb_cut = c->ctl.thb_cut, thb_cutsq = c->ctl.thb_cutsq;
  double e_ang_s = 0, e_pen_s = 0, e_coa_s = 0, e_tor_s = 0, e_con_s = 0;
  int j;
  for (j = 0; j < c->n; j++) { /* valence and torsion both require j < n */
    int tj = c->te[j];
    int start_j = c->b_start[j], end_j = c->b_end[j];
    if (end_j <= start_j) continue;
    double Delta_j = c->bo_dboc1[j];
    double p_val3 = ff->sbp[tj].p_val3, p_val5 = ff->sbp[tj].p_val5;
    double SBOp = 0, prod_SBO = 1, vlpadj, dSBO2, SBO, dSBO1, SBO2, CSBO2;
    int t, pk, ph, pw;
    for (t = start_j; t < end_j; t++) {
      const bond_t *b = &c->bonds[t];
      SBOp += (b->BO_pi + b->BO_pi2);
      double temp = SQR(b->BO);
      temp *= temp;
      temp *= temp;
      prod_SBO *= exp(-temp);
    }
    if (c->vlpex[j] >= 0) {
      vlpadj = 0;
      dSBO2 = prod_SBO - 1;
    } else {
      vlpadj = c->nlp[j];
      dSBO2 = (prod_SBO - 1) * (1 - p_val8 * c->dDelta_lp[j]);
    }
    SBO = SBOp + (1 - prod_SBO) * (-c->bo_dboc1[j] - p_val8 * vlpadj);
    dSBO1 = -8 * prod_SBO * (c->bo_dboc1[j] + p_val8 * vlpadj);
    if (SBO <= 0) SBO2 = 0, CSBO2 = 0;
    else if (SBO > 0 && SBO <= 1) {
      SBO2 = pow(SBO, p_val9);
      CSBO2 = p_val9 * pow(SBO, p_val9 - 1);
    } else if (SBO > 1 && SBO < 2) {
      SBO2 = 2 - pow(2 - SBO, p_val9);
      CSBO2 = p_val9 * pow(2 - SBO, p_val9 - 1);
    } else SBO2 = 2, CSBO2 = 0;
    double expval6 = exp(p_val6 * c->bo_dboc1[j]);

    for (pk = start_j; pk < end_j; pk++) {
      bond_t *bjk = &c->bonds[pk];
      int k = bjk->nbr;
      double BOA_jk = bjk->BO - thb_cut;
      if (!(BOA_jk > 0.0)) continue; /* (j < n) always holds here */
      int pj = bjk->sym;
      if (pj < 0) continue;
      bond_t *bpj = &c->bonds[pj];
      int start_k = c->b_start[k], end_k = c->b_end[k];
      if (end_k <= start_k) continue;
      int tk = c->te[k];
      double Delta_k = c->bo_dboc1[k];
      double r_jk = bjk->d;
      double exp_tor2_jk = exp(-p_tor2 * BOA_jk);
      double exp_cot2_jk = exp(-p_cot2 * SQR(BOA_jk - 1.5));
      double exp_tor3_DjDk = exp(-p_tor3 * (Delta_j + Delta_k));
      double exp_tor4_DjDk = exp(p_tor4 * (Delta_j + Delta_k));
      double exp_tor34_inv = 1.0 / (1.0 + exp_tor3_DjDk + exp_tor4_DjDk);
      double f11_DjDk = (2.0 + exp_tor3_DjDk) * exp_tor34_inv;
      for (ph = start_j; ph < end_j; ph++) {
        if (ph == pk) continue;
        bond_t *bhj = &c->bonds[ph];
        double BOA_hj = bhj->BO - thb_cut;
        int h = bhj->nbr, th = c->te[h];
        thb_t p_hjk;
        double theta_hjk, cos_theta_hjk;
        calc_theta(bjk->dvec, bjk->d, bhj->dvec, bhj->d, &theta_hjk, &cos_theta_hjk);
        calc_dcos_theta(bjk->dvec, bjk->d, bhj->dvec, bhj->d, p_hjk.dcos_di,
                        p_hjk.dcos_dj, p_hjk.dcos_dk);
        p_hjk.theta = theta_hjk;
        double sin_theta_hjk = sin(theta_hjk);
        if (sin_theta_hjk < 1.0e-5) sin_theta_hjk = 1.0e-5;
        /* valence */
        if (ph > pk && bjk->BO > thb_cut && bhj->BO > thb_cut &&
            bjk->BO * bhj->BO > thb_cutsq) {
          const thbh_t *thbh = &ff->thbp[tk][tj][th];
          int cnt;
          for (cnt = 0; cnt < thbh->cnt; cnt++) {
            const thbp_t *thbp = &thbh->prm[cnt];
            if (!(fabs(thbp->p_val1) > 0.001)) continue;
            double p_val1 = thbp->p_val1, p_val2 = thbp->p_val2;
            double p_val4 = thbp->p_val4, p_val7 = thbp->p_val7;
            double theta_00 = thbp->theta_00;
            double exp3jk = exp(-p_val3 * pow(BOA_jk, p_val4));
            double f7_jk = 1.0 - exp3jk;
            double Cf7jk = p_val3 * p_val4 * pow(BOA_jk, p_val4 - 1.0) * exp3jk;
            double exp3hj = exp(-p_val3 * pow(BOA_hj, p_val4));
            double f7_hj = 1.0 - exp3hj;
            double Cf7hj = p_val3 * p_val4 * pow(BOA_hj, p_val4 - 1.0) * exp3hj;
            double expval7 = exp(-p_val7 * c->bo_dboc1[j]);
            double trm8 = 1.0 + expval6 + expval7;
            double f8_Dj = p_val5 - ((p_val5 - 1.0) * (2.0 + expval6) / trm8);
            double Cf8j = ((1.0 - p_val5) / SQR(trm8)) *
                          (p_val6 * expval6 * trm8 -
                           (2.0 + expval6) * (p_val6 * expval6 - p_val7 * expval7));
            double theta_0 = 180.0 - theta_00 * (1.0 - exp(-p_val10 * (2.0 - SBO2)));
            theta_0 = DEG2RAD(theta_0);
            double expval2theta = exp(-p_val2 * SQR(theta_0 - theta_hjk));
            double expval12theta;
            if (p_val1 >= 0) expval12theta = p_val1 * (1.0 - expval2theta);
            else expval12theta = p_val1 * -expval2theta;
            double CEval1 = Cf7jk * f7_hj * f8_Dj * expval12theta;
            double CEval2 = Cf7hj * f7_jk * f8_Dj * expval12theta;
            double CEval3 = Cf8j * f7_hj * f7_jk * expval12theta;
            double CEval4 = -2.0 * p_val1 * p_val2 * f7_jk * f7_hj * f8_Dj *
                            expval2theta * (theta_0 - theta_hjk);
            double Ctheta_0 = p_val10 * DEG2RAD(theta_00) * exp(-p_val10 * (2.0 - SBO2));
            double CEval5 = -CEval4 * Ctheta_0 * CSBO2;
            double CEval6 = CEval5 * dSBO1;
            double CEval7 = CEval5 * dSBO2;
            double CEval8 = -CEval4 / sin_theta_hjk;
            double e_ang = f7_jk * f7_hj * f8_Dj * expval12theta;
            e_ang_s += e_ang;
            double p_pen1 = thbp->p_pen1;
            double exp_pen2jk = exp(-p_pen2 * SQR(BOA_jk - 2.0));
            double exp_pen2hj = exp(-p_pen2 * SQR(BOA_hj - 2.0));
            double exp_pen3 = exp(-p_pen3 * c->Delta[j]);
            double exp_pen4 = exp(p_pen4 * c->Delta[j]);
            double trm_pen34 = 1.0 + exp_pen3 + exp_pen4;
            double f9_Dj = (2.0 + exp_pen3) / trm_pen34;
            double Cf9j = (-p_pen3 * exp_pen3 * trm_pen34 -
                           (2.0 + exp_pen3) * (-p_pen3 * exp_pen3 + p_pen4 * exp_pen4)) /
                          SQR(trm_pen34);
            double e_pen = p_pen1 * f9_Dj * exp_pen2jk * exp_pen2hj;
            e_pen_s += e_pen;
            double CEpen1 = e_pen * Cf9j / f9_Dj;
            double temp = -2.0 * p_pen2 * e_pen;
            double CEpen2 = temp * (BOA_jk - 2.0);
            double CEpen3 = temp * (BOA_hj - 2.0);
            double p_coa1 = thbp->p_coa1;
            double exp_coa2 = exp(p_coa2 * c->Delta_val[j]);
            double e_coa = p_coa1 / (1. + exp_coa2) *
                           exp(-p_coa3 * SQR(c->bo_dboc0[k] - BOA_jk)) *
                           exp(-p_coa3 * SQR(c->bo_dboc0[h] - BOA_hj)) *
                           exp(-p_coa4 * SQR(BOA_jk - 1.5)) *
                           exp(-p_coa4 * SQR(BOA_hj - 1.5));
            e_coa_s += e_coa;
            double CEcoa1 = -2 * p_coa4 * (BOA_jk - 1.5) * e_coa;
            double CEcoa2 = -2 * p_coa4 * (BOA_hj - 1.5) * e_coa;
            double CEcoa3 = -p_coa2 * exp_coa2 * e_coa / (1 + exp_coa2);
            double CEcoa4 = -2 * p_coa3 * (c->bo_dboc0[k] - BOA_jk) * e_coa;
            double CEcoa5 = -2 * p_coa3 * (c->bo_dboc0[h] - BOA_hj) * e_coa;
            bjk->Cdbo += (CEval1 + CEpen2 + (CEcoa1 - CEcoa4));
            bhj->Cdbo += (CEval2 + CEpen3 + (CEcoa2 - CEcoa5));
            c->fC[4 * j + 3] += ((CEval3 + CEval7) + CEpen1 + CEcoa3);
            c->fC[4 * k + 3] += CEcoa4;
            c->fC[4 * h + 3] += CEcoa5;
            for (t = start_j; t < end_j; t++) {
              bond_t *bjt = &c->bonds[t];
              double temp_bo_jt = bjt->BO;
              double tmp3 = CUBE(temp_bo_jt);
              double pBOjt7 = tmp3 * tmp3 * temp_bo_jt;
              bjt->Cdbo += (CEval6 * pBOjt7);
              bjt->Cdbopi += CEval5;
              bjt->Cdbopi2 += CEval5;
            }
            add4(&c->fC[4 * k], CEval8, p_hjk.dcos_di);
            add4(&c->fC[4 * j], CEval8, p_hjk.dcos_dj);
            add4(&c->fC[4 * h], CEval8, p_hjk.dcos_dk);
          }
        }
        /* torsion: central bond counted once (tag order), :1135-1146 */
        if (!tag_first(c, j, k)) continue;
        if (bhj->BO > thb_cut && end_k > start_k) {
          int i = h, ti = th;
          double r_ij = bhj->d;
          double BOA_ij = bhj->BO - thb_cut;
          double theta_ijk = p_hjk.theta;
          double sin_ijk = sin(theta_ijk), cos_ijk = cos(theta_ijk), tan_ijk_i;
          if (sin_ijk >= 0 && sin_ijk <= MIN_SINE) tan_ijk_i = cos_ijk / MIN_SINE;
          else if (sin_ijk <= 0 && sin_ijk >= -MIN_SINE) tan_ijk_i = cos_ijk / -MIN_SINE;
          else tan_ijk_i = cos_ijk / sin_ijk;
          double exp_tor2_ij = exp(-p_tor2 * BOA_ij);
          double exp_cot2_ij = exp(-p_cot2 * SQR(BOA_ij - 1.5));
          for (pw = start_k; pw < end_k; pw++) {
            if (pw == pj) continue;
            bond_t *bkl = &c->bonds[pw];
            int l = bkl->nbr, tl = c->te[l];
            thb_t p_jkl;
            double theta_jkl, cos_theta_jkl;
            calc_theta(bpj->dvec, bpj->d, bkl->dvec, bkl->d, &theta_jkl, &cos_theta_jkl);
            calc_dcos_theta(bpj->dvec, bpj->d, bkl->dvec, bkl->d, p_jkl.dcos_di,
                            p_jkl.dcos_dj, p_jkl.dcos_dk);
            p_jkl.theta = theta_jkl;
            const fbh_t *fbh = &ff->fbp[ti][tj][tk][tl];
            const fbp_t *fbp = &fbh->prm;
            if (i != l && fbh->cnt && bkl->BO > thb_cut &&
                bhj->BO * bjk->BO * bkl->BO > thb_cut) {
              double r_kl = bkl->d;
              double BOA_kl = bkl->BO - thb_cut;
              double sin_jkl = sin(theta_jkl), cos_jkl = cos(theta_jkl), tan_jkl_i;
              if (sin_jkl >= 0 && sin_jkl <= MIN_SINE) tan_jkl_i = cos_jkl / MIN_SINE;
              else if (sin_jkl <= 0 && sin_jkl >= -MIN_SINE) tan_jkl_i = cos_jkl / -MIN_SINE;
              else tan_jkl_i = cos_jkl / sin_jkl;
              double dvec_li[3];
              dvec_li[0] = c->xe[3 * i + 0] - c->xe[3 * l + 0];
              dvec_li[1] = c->xe[3 * i + 1] - c->xe[3 * l + 1];
              dvec_li[2] = c->xe[3 * i + 2] - c->xe[3 * l + 2];
              double r_li = sqrt(SQR(dvec_li[0]) + SQR(dvec_li[1]) + SQR(dvec_li[2]));
              double dcos_omega_di[3], dcos_omega_dj[3], dcos_omega_dk[3], dcos_omega_dl[3];
              double omega = calc_omega(bhj->dvec, r_ij, bjk->dvec, r_jk, bkl->dvec, r_kl,
                                        dvec_li, r_li, &p_hjk, &p_jkl, dcos_omega_di,
                                        dcos_omega_dj, dcos_omega_dk, dcos_omega_dl);
              double cos_omega = cos(omega);
              double cos2omega = cos(2. * omega);
              double cos3omega = cos(3. * omega);
              double exp_tor1 = exp(fbp->p_tor1 * SQR(2.0 - bjk->BO_pi - f11_DjDk));
              double exp_tor2_kl = exp(-p_tor2 * BOA_kl);
              double exp_cot2_kl = exp(-p_cot2 * SQR(BOA_kl - 1.5));
              double fn10 = (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
              double CV = 0.5 * (fbp->V1 * (1.0 + cos_omega) +
                                 fbp->V2 * exp_tor1 * (1.0 - cos2omega) +
                                 fbp->V3 * (1.0 + cos3omega));
              double e_tor = fn10 * sin_ijk * sin_jkl * CV;
              e_tor_s += e_tor;
              double dfn11 = (-p_tor3 * exp_tor3_DjDk +
                              (p_tor3 * exp_tor3_DjDk - p_tor4 * exp_tor4_DjDk) *
                                  (2.0 + exp_tor3_DjDk) * exp_tor34_inv) *
                             exp_tor34_inv;
              double CEtors1 = sin_ijk * sin_jkl * CV;
              double CEtors2 = -fn10 * 2.0 * fbp->p_tor1 * fbp->V2 * exp_tor1 *
                               (2.0 - bjk->BO_pi - f11_DjDk) * (1.0 - SQR(cos_omega)) *
                               sin_ijk * sin_jkl;
              double CEtors3 = CEtors2 * dfn11;
              double CEtors4 = CEtors1 * p_tor2 * exp_tor2_ij * (1.0 - exp_tor2_jk) * (1.0 - exp_tor2_kl);
              double CEtors5 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * exp_tor2_jk * (1.0 - exp_tor2_kl);
              double CEtors6 = CEtors1 * p_tor2 * (1.0 - exp_tor2_ij) * (1.0 - exp_tor2_jk) * exp_tor2_kl;
              double cmn = -fn10 * CV;
              double CEtors7 = cmn * sin_jkl * tan_ijk_i;
              double CEtors8 = cmn * sin_ijk * tan_jkl_i;
              double CEtors9 = fn10 * sin_ijk * sin_jkl *
                               (0.5 * fbp->V1 - 2.0 * fbp->V2 * exp_tor1 * cos_omega +
                                1.5 * fbp->V3 * (cos2omega + 2.0 * SQR(cos_omega)));
              double fn12 = exp_cot2_ij * exp_cot2_jk * exp_cot2_kl;
              double e_con = fbp->p_cot1 * fn12 * (1.0 + (SQR(cos_omega) - 1.0) * sin_ijk * sin_jkl);
              e_con_s += e_con;
              double Cconj = -2.0 * fn12 * fbp->p_cot1 * p_cot2 *
                             (1.0 + (SQR(cos_omega) - 1.0) * sin_ijk * sin_jkl);
              double CEconj1 = Cconj * (BOA_ij - 1.5e0);
              double CEconj2 = Cconj * (BOA_jk - 1.5e0);
              double CEconj3 = Cconj * (BOA_kl - 1.5e0);
              double CEconj4 = -fbp->p_cot1 * fn12 * (SQR(cos_omega) - 1.0) * sin_jkl * tan_ijk_i;
              double CEconj5 = -fbp->p_cot1 * fn12 * (SQR(cos_omega) - 1.0) * sin_ijk * tan_jkl_i;
              double CEconj6 = 2.0 * fbp->p_cot1 * fn12 * cos_omega * sin_ijk * sin_jkl;
              bjk->Cdbopi += CEtors2;
              c->fC[4 * j + 3] += CEtors3;
              c->fC[4 * k + 3] += CEtors3;
              bhj->Cdbo += (CEtors4 + CEconj1);
              bjk->Cdbo += (CEtors5 + CEconj2);
              bkl->Cdbo += (CEtors6 + CEconj3);
              add4(&c->fC[4 * i], CEtors7 + CEconj4, p_hjk.dcos_dk);
              add4(&c->fC[4 * j], CEtors7 + CEconj4, p_hjk.dcos_dj);
              add4(&c->fC[4 * k], CEtors7 + CEconj4, p_hjk.dcos_di);
              add4(&c->fC[4 * j], CEtors8 + CEconj5, p_jkl.dcos_di);
              add4(&c->fC[4 * k], CEtors8 + CEconj5, p_jkl.dcos_dj);
              add4(&c->fC[4 * l], CEtors8 + CEconj5, p_jkl.dcos_dk);
              add4(&c->fC[4 * i], CEtors9 + CEconj6, dcos_omega_di);
              add4(&c->fC[4 * j], CEtors9 + CEconj6, dcos_omega_dj);
              add4(&c->fC[4 * k], CEtors9 + CEconj6, dcos_omega_dk);
              add4(&c->fC[4 * l], CEtors9 + CEconj6, dcos_omega_dl);
            }
          }
        }
      }
    }
  }
  c->en[RO_E_ANG] += e_ang_s;
  c->en[RO_E_PEN] += e_pen_s;
  c->en[RO_E_COA] += e_coa_s;
  c->en[RO_E_TOR] += e_tor_s;
  c->en[RO_E_CON] += e_con_s;
  c->en[RO_ENG_VDWL] += e_ang_s + e_pen_s + e_coa_s + e_tor_s + e_con_s;
}

/* ------------------------------------------------------------------ */
/* vdW + Coulomb, full list, forces on i only:
 * vdW_Coulomb_Energy_Full_C_test_err, reaxc_nonbonded_sw64.c:40-258 */

static void tally_alloc(ro_ctx *c) {
  if (c->tally_n != c->n) {
    free(c->eatom); free(c->vatom); free(c->ref_eatom); free(c->ref_vatom);
    c->eatom = (double *)calloc((size_t)c->n + 1, sizeof(double));
    c->vatom = (double *)calloc(6 * (size_t)c->n + 1, sizeof(double));
    c->ref_eatom = (double *)calloc((size_t)c->n + 1, sizeof(double));
    c->ref_vatom = (double *)calloc(6 * (size_t)c->n + 1, sizeof(double));
    c->tally_n = c->n;
  }
}

static void nonbonded(ro_ctx *c) {
  const ffield_t *ff = &c->ff;
  const double p_vdW1 = ff->gp[28], p_vdW1i = 1.0 / p_vdW1;
  const double *Tap = c->Tap;
  double e_vdw_full = 0, e_ele_full = 0, eng_vdwl = 0, eng_coul = 0;
  int i;
  tally_alloc(c);
  memset(c->eatom, 0, (size_t)c->n * sizeof(double));
  memset(c->vatom, 0, 6 * (size_t)c->n * sizeof(double));
  for (i = 0; i < c->n; i++) {
    int ti = c->te[i], pj;
    for (pj = c->far_start[i]; pj < c->far_start[i + 1]; pj++) {
      int j = c->far_nbr[pj], tj = c->te[j];
      double r_ij = c->far_d[pj];
      const tbp_t *tw = &ff->tbp[ti][tj];
      double Tp = Tap[7] * r_ij + Tap[6];
      Tp = Tp * r_ij + Tap[5];
      Tp = Tp * r_ij + Tap[4];
      Tp = Tp * r_ij + Tap[3];
      Tp = Tp * r_ij + Tap[2];
      Tp = Tp * r_ij + Tap[1];
      Tp = Tp * r_ij + Tap[0];
      double dTap = 7 * Tap[7] * r_ij + 6 * Tap[6];
      dTap = dTap * r_ij + 5 * Tap[5];
      dTap = dTap * r_ij + 4 * Tap[4];
      dTap = dTap * r_ij + 3 * Tap[3];
      dTap = dTap * r_ij + 2 * Tap[2];
      dTap += Tap[1] / r_ij;
      double e_vdW, CEvd, e_core = 0, e_lg = 0;
      if (ff->vdw_type == 1 || ff->vdw_type == 3) {
        double powr_vdW1 = pow(r_ij, p_vdW1);
        double powgi_vdW1 = pow(1.0 / tw->gamma_w, p_vdW1);
        double fn13 = pow(powr_vdW1 + powgi_vdW1, p_vdW1i);
        double exp1 = exp(tw->alpha * (1.0 - fn13 / tw->r_vdW));
        double exp2 = exp(0.5 * tw->alpha * (1.0 - fn13 / tw->r_vdW));
        e_vdW = tw->D * (exp1 - 2.0 * exp2);
        double dfn13 = pow(powr_vdW1 + powgi_vdW1, p_vdW1i - 1.0) * pow(r_ij, p_vdW1 - 2.0);
        CEvd = dTap * e_vdW - Tp * tw->D * (tw->alpha / tw->r_vdW) * (exp1 - exp2) * dfn13;
      } else {
        double exp1 = exp(tw->alpha * (1.0 - r_ij / tw->r_vdW));
        double exp2 = exp(0.5 * tw->alpha * (1.0 - r_ij / tw->r_vdW));
        e_vdW = tw->D * (exp1 - 2.0 * exp2);
        CEvd = dTap * e_vdW - Tp * tw->D * (tw->alpha / tw->r_vdW) * (exp1 - exp2) / r_ij;
      }
      e_vdw_full += Tp * e_vdW;
      if (ff->vdw_type == 2 || ff->vdw_type == 3) {
        e_core = tw->ecore * exp(tw->acore * (1.0 - (r_ij / tw->rcore)));
        e_vdw_full += Tp * e_core;
        double de_core = -(tw->acore / tw->rcore) * e_core;
        CEvd += dTap * e_core + Tp * de_core / r_ij;
        if (c->ctl.lgflag) {
          double r_ij5 = pow(r_ij, 5.0), r_ij6 = pow(r_ij, 6.0);
          double re6 = pow(tw->lgre, 6.0);
          e_lg = -(tw->lgcij / (r_ij6 + re6));
          e_vdw_full += Tp * e_lg;
          double de_lg = -6.0 * e_lg * r_ij5 / (r_ij6 + re6);
          CEvd += dTap * e_lg + Tp * de_lg / r_ij;
        }
      }
      double dr3gamij_1 = (r_ij * r_ij * r_ij + tw->gamma);
      double dr3gamij_3 = pow(dr3gamij_1, 0.33333333333333);
      double tmp = Tp / dr3gamij_3;
      double qi = c->q[c->own[i]], qj = c->q[c->own[j]];
      double e_ele = C_ele * qi * qj * tmp;
      e_ele_full += e_ele;
      double CEclmb = C_ele * qi * qj * (dTap - Tp * r_ij / dr3gamij_1) / dr3gamij_3;
      eng_vdwl += 0.5 * Tp * (e_vdW + e_core + e_lg);
      eng_coul += 0.5 * e_ele;
      add4(&c->fC[4 * i], -(CEvd + CEclmb), &c->far_dvec[3 * pj]);
      {
        /* per-atom tallies: ev_tally_full (reaxc_inlines_sw64.h:178-222)
         * as called at reaxc_nonbonded_sw64.c:198-213, del = x_i - x_j of
         * the ghost positions, fpair = -(CEvd + CEclmb) */
        const double pe_vdw = Tp * (e_vdW + e_core + e_lg);
        const double f_tmp = -(CEvd + CEclmb);
        const double dx = c->xe[3 * i] - c->xe[3 * j], dy = c->xe[3 * i + 1] - c->xe[3 * j + 1],
                     dz = c->xe[3 * i + 2] - c->xe[3 * j + 2];
        double *va = &c->vatom[6 * i];
        c->eatom[i] += 0.5 * (pe_vdw + e_ele);
        va[0] += 0.5 * dx * dx * f_tmp;
        va[1] += 0.5 * dy * dy * f_tmp;
        va[2] += 0.5 * dz * dz * f_tmp;
        va[3] += 0.5 * dx * dy * f_tmp;
        va[4] += 0.5 * dx * dz * f_tmp;
        va[5] += 0.5 * dy * dz * f_tmp;
      }
    }
  }
  c->en[RO_E_VDW] += e_vdw_full;
  c->en[RO_E_ELE] += e_ele_full;
  c->en[RO_ENG_VDWL] += eng_vdwl;
  c->en[RO_ENG_COUL] += eng_coul;
}

/* ------------------------------------------------------------------ */
/* bond-order derivative forces: Add_All_dBond_to_Forces_C CPU form,
 * reaxc_forces_sw64.c:499-588 */

static void dbond_forces(ro_ctx *c) {
  int i, N = c->N;
  int *buf_idx = NULL;
  double *buf_dBOp = NULL;
  int bufcap = 0;
  for (i = 0; i < N; i++) {
    int s = c->b_start[i], e = c->b_end[i], pj;
    if (e - s > bufcap) {
      bufcap = e - s + 16;
      buf_idx = (int *)xrealloc(buf_idx, bufcap * sizeof(int));
      buf_dBOp = (double *)xrealloc(buf_dBOp, bufcap * 3 * sizeof(double));
    }
    double buf_c = 0.0;
    const double *dDi = &c->dDeltap_self[3 * i];
    for (pj = s; pj < e; pj++) {
      const bond_t *b = &c->bonds[pj];
      int j = b->nbr;
      double cdbo = b->Cdbo, cdbopi = b->Cdbopi, cdbopi2 = b->Cdbopi2;
      if (b->sym >= 0) {
        const bond_t *bs = &c->bonds[b->sym];
        cdbo += bs->Cdbo;
        cdbopi += bs->Cdbopi;
        cdbopi2 += bs->Cdbopi2;
      }
      double C1dbo = b->C1dbo * cdbo, C2dbo = b->C2dbo * cdbo;
      double C1dbopi = b->C1dbopi * cdbopi, C2dbopi = b->C2dbopi * cdbopi;
      double C3dbopi = b->C3dbopi * cdbopi;
      double C1dbopi2 = b->C1dbopi2 * cdbopi2, C2dbopi2 = b->C2dbopi2 * cdbopi2;
      double C3dbopi2 = b->C3dbopi2 * cdbopi2;
      double cdd = c->fC[4 * i + 3] + c->fC[4 * j + 3];
      double C1dDelta = b->C1dbo * cdd, C2dDelta = b->C2dbo * cdd;
      int t;
      for (t = 0; t < 3; t++) {
        double temp = C1dbo * b->dBOp[t];
        temp += C2dbo * dDi[t];
        temp += C1dDelta * b->dBOp[t];
        temp += C2dDelta * dDi[t];
        temp += C1dbopi * b->dln_BOp_pi[t];
        temp += C2dbopi * b->dBOp[t];
        temp += C3dbopi * dDi[t];
        temp += C1dbopi2 * b->dln_BOp_pi2[t];
        temp += C2dbopi2 * b->dBOp[t];
        temp += C3dbopi2 * dDi[t];
        c->fC[4 * i + t] += temp;
      }
      buf_c += (-C2dbo - C2dDelta - C3dbopi - C3dbopi2);
      buf_dBOp[3 * (pj - s) + 0] = b->dBOp[0];
      buf_dBOp[3 * (pj - s) + 1] = b->dBOp[1];
      buf_dBOp[3 * (pj - s) + 2] = b->dBOp[2];
      buf_idx[pj - s] = j;
    }
    for (pj = s; pj < e; pj++) add4(&c->fC[4 * buf_idx[pj - s]], buf_c, &buf_dBOp[3 * (pj - s)]);
  }
  free(buf_idx);
  free(buf_dBOp);
}

/* ------------------------------------------------------------------ */

static void prepare_lists(ro_ctx *c) {
  double t0 = now_s();
  build_ghosts(c);
  build_far(c);
  c->tphase[0] += now_s() - t0;
}

int ro_compute(ro_ctx *c, double *f_out, double *energies) {
  int i, k;
  double t0;
  prepare_lists(c);
  t0 = now_s();
  build_bonds(c);
  build_hbonds(c);
  c->tphase[1] += now_s() - t0;
  for (k = 0; k < RO_NENERGY; k++) c->en[k] = 0;
  for (i = 0; i < 4 * c->N; i++) c->fC[i] = 0;
  t0 = now_s();
  bond_orders(c);
  c->tphase[1] += now_s() - t0;
  t0 = now_s();
  atom_energy(c);
  hydrogen_bonds(c);
  torsion_valence(c);
  c->tphase[2] += now_s() - t0;
  t0 = now_s();
  nonbonded(c);
  c->tphase[3] += now_s() - t0;
  t0 = now_s();
  dbond_forces(c);
  /* copy-out f -= fCdDelta, ghosts folded to owners
   * (pair_reaxc_sunway.cpp:674-702 + LAMMPS reverse comm) */
  for (i = 0; i < 3 * c->n; i++) c->f[i] = 0;
  for (i = 0; i < c->n; i++) c->cd_local[i] = 0;
  for (i = 0; i < c->N; i++) {
    int o = c->own[i];
    c->f[3 * o + 0] -= c->fC[4 * i + 0];
    c->f[3 * o + 1] -= c->fC[4 * i + 1];
    c->f[3 * o + 2] -= c->fC[4 * i + 2];
    c->cd_local[o] += c->fC[4 * i + 3];
  }
  c->tphase[2] += now_s() - t0;
  if (f_out) memcpy(f_out, c->f, 3 * (size_t)c->n * sizeof(double));
  if (energies) memcpy(energies, c->en, sizeof(c->en));
  return 0;
}

/* ------------------------------------------------------------------ */
/* QEq: H rows (compute_H_Full_C CPU form, fix_qeq_reax_sw64.c:146-181),
 * sparse_matvec (fix_qeq_reax_sunway.cpp:1563-1623), pipelined PCG CG_v2
 * (:983-1167), init_matvec extrapolation (:618-723), calculate_Q
 * (:1697-1755).  Ghost columns carry their owner's value (forward comm). */

typedef struct {
  int *start, *col;
  double *val;
} hmat_t;

static void qeq_matvec(const ro_ctx *c, const hmat_t *H, const double *x,
                       double *b) {
  int i, p;
  for (i = 0; i < c->n; i++) {
    double bi = c->ff.sbp[c->type[i]].eta * x[i];
    for (p = H->start[i]; p < H->start[i + 1]; p++) bi += H->val[p] * x[H->col[p]];
    b[i] = bi;
  }
}

static int qeq_cg(const ro_ctx *c, const hmat_t *H, const double *b,
                  double *x, const double *Hdia_inv) {
  int n = c->n, i, jj;
  double *r = (double *)calloc(n, sizeof(double)), *u = (double *)calloc(n, sizeof(double));
  double *d = (double *)calloc(n, sizeof(double)), *q = (double *)calloc(n, sizeof(double));
  double *w = (double *)calloc(n, sizeof(double)), *m = (double *)calloc(n, sizeof(double));
  double *p = (double *)calloc(n, sizeof(double)), *ss = (double *)calloc(n, sizeof(double));
  double *v = (double *)calloc(n, sizeof(double)), *z = (double *)calloc(n, sizeof(double));
  double alpha, beta, b_norm, sig_old, deta, heta, dot0 = 0, dot1 = 0;
  int imax = c->ctl.qeq_imax;
  qeq_matvec(c, H, x, q);
  for (jj = 0; jj < n; jj++) {
    r[jj] = b[jj] - 1 * q[jj];
    u[jj] = r[jj] * Hdia_inv[jj];
    d[jj] = u[jj];
  }
  qeq_matvec(c, H, d, q);
  for (jj = 0; jj < n; jj++) {
    w[jj] = q[jj];
    m[jj] = q[jj] * Hdia_inv[jj];
    d[jj] = m[jj];
  }
  qeq_matvec(c, H, d, q);
  double s0 = 0, s1 = 0, s2 = 0;
  for (jj = 0; jj < n; jj++) {
    p[jj] = u[jj];
    ss[jj] = w[jj];
    v[jj] = m[jj];
    s0 += SQR(b[jj]);
    s1 += u[jj] * r[jj];
    s2 += u[jj] * w[jj];
  }
  b_norm = sqrt(s0);
  sig_old = s1;
  deta = s2;
  heta = deta;
  alpha = sig_old / deta;
  dot0 = sig_old;
  for (jj = 0; jj < n; jj++) z[jj] = q[jj];
  for (i = 1; i < imax && sqrt(dot0) / b_norm > c->ctl.qeq_tol; ++i) {
    dot0 = dot1 = 0.0;
    for (jj = 0; jj < n; jj++) {
      r[jj] -= alpha * ss[jj];
      u[jj] -= alpha * v[jj];
      w[jj] -= alpha * z[jj];
      dot0 += u[jj] * r[jj];
      dot1 += u[jj] * w[jj];
      d[jj] = w[jj] * Hdia_inv[jj];
    }
    qeq_matvec(c, H, d, q);
    beta = dot0 / sig_old;
    heta = dot1 - beta * beta * heta;
    for (jj = 0; jj < n; jj++) {
      x[jj] += alpha * p[jj];
      p[jj] = u[jj] + p[jj] * beta;
      ss[jj] = w[jj] + ss[jj] * beta;
      v[jj] = d[jj] + v[jj] * beta;
    }
    alpha = dot0 / heta;
    for (jj = 0; jj < n; jj++) z[jj] = q[jj] + z[jj] * beta;
    sig_old = dot0;
  }
  free(r); free(u); free(d); free(q); free(w); free(m); free(p); free(ss);
  free(v); free(z);
  return i;
}

/* H rows of the local atoms from the full far list (compute_H_Full_C_para,
 * fix_qeq_reax_sw64.c:768-911, host form :146-181), ghost columns folded
 * onto their local owners */
/* The fix's neighbour list reaches the pair cutoff plus the skin
 * (cutmax + skin, the ghosts' range), and compute_H keeps r <= swb: within
 * nonb_cut that is the far list; for swb > nonb_cut the pairs are searched
 * among all ghosts (a plain loop: such runs are small test cases). */
static void qeq_build_H(ro_ctx *c, hmat_t *H_out) {
  int i, n = c->n;
  const double swbsq = c->ctl.qeq_swb * c->ctl.qeq_swb;
  const int wide = c->ctl.qeq_swb > c->nonb_cut;
  const double *Tap = c->qTap;
  hmat_t H;
  H.start = (int *)malloc((n + 1) * sizeof(int));
  long long cap = wide ? (long long)n * 64 + 16 : c->far_start[n] + 16, top = 0;
  H.col = (int *)malloc(cap * sizeof(int));
  H.val = (double *)malloc(cap * sizeof(double));
  for (i = 0; i < n; i++) {
    int pj, ti = c->type[i];
    H.start[i] = (int)top;
    const int p0 = wide ? 0 : c->far_start[i], p1 = wide ? c->N : c->far_start[i + 1];
    for (pj = p0; pj < p1; pj++) {
      int j;
      double dvw[3];
      const double *dv;
      if (wide) {
        j = pj;
        if (j == i) continue;
        dvw[0] = c->xe[3 * j + 0] - c->xe[3 * i + 0];
        dvw[1] = c->xe[3 * j + 1] - c->xe[3 * i + 1];
        dvw[2] = c->xe[3 * j + 2] - c->xe[3 * i + 2];
        dv = dvw;
      } else {
        j = c->far_nbr[pj];
        dv = &c->far_dvec[3 * pj];
      }
      double r_sqr = SQR(dv[0]) + SQR(dv[1]) + SQR(dv[2]);
      if (r_sqr <= swbsq) {
        if (top >= cap) {
          cap *= 2;
          H.col = (int *)xrealloc(H.col, cap * sizeof(int));
          H.val = (double *)xrealloc(H.val, cap * sizeof(double));
        }
        double r = sqrt(r_sqr);
        /* shld = pow(gamma_i*gamma_j, -1.5), init_shielding :440-454 */
        double gamma = pow(c->ff.sbp[ti].gamma * c->ff.sbp[c->te[j]].gamma, -1.5);
        double Taper = Tap[7] * r + Tap[6];
        Taper = Taper * r + Tap[5];
        Taper = Taper * r + Tap[4];
        Taper = Taper * r + Tap[3];
        Taper = Taper * r + Tap[2];
        Taper = Taper * r + Tap[1];
        Taper = Taper * r + Tap[0];
        double denom = r * r * r + gamma;
        denom = pow(denom, 0.3333333333333);
        H.col[top] = c->own[j];
        H.val[top] = Taper * EV_TO_KCAL_PER_MOL / denom;
        top++;
      }
    }
  }
  H.start[n] = (int)top;
  c->H_entries = top;
  *H_out = H;
}

/* init_matvec's extrapolation, CG_v2 on s and t, calculate_Q
 * (fix_qeq_reax_sunway.cpp:539-600, 618-723, 983-1167, 1697-1755) */
static int qeq_restated(ro_ctx *c, const hmat_t *Hp, int *iters_s, int *iters_t) {
  int i, n = c->n, k;
  const hmat_t H = *Hp;
  double *Hdia_inv = (double *)malloc(n * sizeof(double));
  double *b_s = (double *)malloc(n * sizeof(double));
  double *b_t = (double *)malloc(n * sizeof(double));
  for (i = 0; i < n; i++) {
    const sbp_t *s = &c->ff.sbp[c->type[i]];
    Hdia_inv[i] = 1. / s->eta;
    b_s[i] = -s->chi;
    b_t[i] = -1.0;
    const double *sh = &c->s_hist[5 * i], *th = &c->t_hist[5 * i];
    c->t[i] = th[2] + 3 * (th[0] - th[1]);
    c->s[i] = 4 * (sh[0] + sh[2]) - (6 * sh[1] + sh[3]);
  }
  int is = qeq_cg(c, &H, b_s, c->s, Hdia_inv);
  int it = qeq_cg(c, &H, b_t, c->t, Hdia_inv);
  double s_sum = 0, t_sum = 0;
  for (i = 0; i < n; i++) {
    s_sum += c->s[i];
    t_sum += c->t[i];
  }
  double u = s_sum / t_sum;
  for (i = 0; i < n; i++) {
    c->q[i] = c->s[i] - u * c->t[i];
    for (k = 4; k > 0; --k) {
      c->s_hist[5 * i + k] = c->s_hist[5 * i + k - 1];
      c->t_hist[5 * i + k] = c->t_hist[5 * i + k - 1];
    }
    c->s_hist[5 * i] = c->s[i];
    c->t_hist[5 * i] = c->t[i];
  }
  free(Hdia_inv); free(b_s); free(b_t);
  if (iters_s) *iters_s = is;
  if (iters_t) *iters_t = it;
  return 0;
}

int ro_qeq(ro_ctx *c, double *q_out, int *iters_s, int *iters_t) {
  hmat_t H;
  double t0;
  int rc;
  prepare_lists(c);
  t0 = now_s();
  qeq_build_H(c, &H);
  rc = c->qeq_driver ? c->qeq_driver(c, &H, iters_s, iters_t)
                     : qeq_restated(c, &H, iters_s, iters_t);
  free(H.start); free(H.col); free(H.val);
  if (q_out) memcpy(q_out, c->q, c->n * sizeof(double));
  c->tphase[4] += now_s() - t0;
  return rc;
}

/* ------------------------------------------------------------------ */
/* NVE: fix_nve_sw64.c:25-172 (velocity Verlet, dtf = 0.5*dt*ftm2v,
 * fix_nve_sunway.cpp:54-58), Verlet order initial_integrate -> pre_force
 * (QEq) -> compute -> final_integrate */

int ro_run_nve(ro_ctx *c, int nsteps, double dt, double *energies_last) {
  ro_qeq(c, NULL, NULL, NULL);
  ro_compute(c, NULL, energies_last);
  return ro_md_steps(c, nsteps, dt, energies_last);
}

int ro_md_steps(ro_ctx *c, int nsteps, double dt, double *energies_last) {
  int step, i, d;
  const double dtf = 0.5 * dt * FTM2V;
  for (step = 0; step < nsteps; step++) {
    double t0 = now_s();
    for (i = 0; i < c->n; i++) {
      double dtfm = dtf / c->ff.sbp[c->type[i]].mass;
      for (d = 0; d < 3; d++) {
        c->v[3 * i + d] += dtfm * c->f[3 * i + d];
        c->x[3 * i + d] += dt * c->v[3 * i + d];
      }
      wrap_pos(c, c->x + 3 * i);
    }
    c->tphase[5] += now_s() - t0;
    ro_qeq(c, NULL, NULL, NULL);
    ro_compute(c, NULL, energies_last);
    t0 = now_s();
    for (i = 0; i < c->n; i++) {
      double dtfm = dtf / c->ff.sbp[c->type[i]].mass;
      for (d = 0; d < 3; d++) c->v[3 * i + d] += dtfm * c->f[3 * i + d];
    }
    c->tphase[5] += now_s() - t0;
  }
  return 0;
}

void ro_atom_tallies(const ro_ctx *c, double *eatom, double *vatom) {
  size_t n = (size_t)c->n;
  if (c->tally_n != c->n) return;
  if (eatom) memcpy(eatom, c->eatom, n * sizeof(double));
  if (vatom) memcpy(vatom, c->vatom, 6 * n * sizeof(double));
}

void ro_get_state(const ro_ctx *c, double *x, double *v, double *q, double *f) {
  size_t n = (size_t)c->n;
  if (x) memcpy(x, c->x, 3 * n * sizeof(double));
  if (v) memcpy(v, c->v, 3 * n * sizeof(double));
  if (q) memcpy(q, c->q, n * sizeof(double));
  if (f) memcpy(f, c->f, 3 * n * sizeof(double));
}

void ro_get_stats(const ro_ctx *c, ro_stats *s) {
  int i;
  memset(s, 0, sizeof *s);
  s->n_local = c->n;
  s->n_total = c->N;
  s->n_far_total = c->far_start ? c->far_start[c->N] : 0;
  s->n_far_local = c->far_start ? c->far_start[c->n] : 0;
  if (c->b_start) {
    for (i = 0; i < c->N; i++) s->n_bonds_total += c->b_end[i] - c->b_start[i];
    for (i = 0; i < c->n; i++) s->n_bonds_local += c->b_end[i] - c->b_start[i];
  }
  s->n_hbonds = c->hb_start ? c->hb_start[c->n] : 0;
  s->n_H_entries = c->H_entries;
}

static int rel_img(const ro_ctx *c, int i, int j) {
  /* image of j relative to i's owner: i is local here so its image is 0 */
  (void)i;
  return c->imgc[j];
}

long long ro_dump_far(const ro_ctx *c, int *ti, int *tj, int *img) {
  long long k = 0;
  int i, p;
  for (i = 0; i < c->n; i++)
    for (p = c->far_start[i]; p < c->far_start[i + 1]; p++, k++)
      if (ti) {
        int j = c->far_nbr[p];
        ti[k] = c->tag[i];
        tj[k] = c->tag[c->own[j]];
        img[k] = rel_img(c, i, j);
      }
  return k;
}

long long ro_dump_bonds(const ro_ctx *c, int *ti, int *tj, int *img,
                        double *bo) {
  long long k = 0;
  int i, p;
  for (i = 0; i < c->n; i++)
    for (p = c->b_start[i]; p < c->b_end[i]; p++, k++)
      if (ti) {
        const bond_t *b = &c->bonds[p];
        ti[k] = c->tag[i];
        tj[k] = c->tag[c->own[b->nbr]];
        img[k] = rel_img(c, i, b->nbr);
        if (bo) {
          bo[4 * k + 0] = b->BO;
          bo[4 * k + 1] = b->BO_s;
          bo[4 * k + 2] = b->BO_pi;
          bo[4 * k + 3] = b->BO_pi2;
        }
      }
  return k;
}

long long ro_dump_hbonds(const ro_ctx *c, int *ti, int *tj, int *img) {
  long long k = 0;
  int i, p;
  for (i = 0; i < c->n; i++)
    for (p = c->hb_start[i]; p < c->hb_start[i + 1]; p++, k++)
      if (ti) {
        int j = c->far_nbr[c->hb_far[p]];
        ti[k] = c->tag[i];
        tj[k] = c->tag[c->own[j]];
        img[k] = rel_img(c, i, j);
      }
  return k;
}

void ro_dump_atom_terms(const ro_ctx *c, double *out) {
  int i;
  for (i = 0; i < c->n; i++) {
    out[8 * i + 0] = c->Deltap[i];
    out[8 * i + 1] = c->Delta[i];
    out[8 * i + 2] = c->Delta_e[i];
    out[8 * i + 3] = c->bo_dboc1[i];
    out[8 * i + 4] = c->Delta_val[i];
    out[8 * i + 5] = c->Delta_lp[i];
    out[8 * i + 6] = c->nlp[i];
    out[8 * i + 7] = c->cd_local[i];
  }
}

double ro_last_time(const ro_ctx *c, int phase) {
  return (phase >= 0 && phase < 8) ? c->tphase[phase] : 0.0;
}
