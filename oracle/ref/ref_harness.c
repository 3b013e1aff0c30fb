/*
 * Reference harness -- TEST INFRASTRUCTURE ONLY, built only where the
 * reference sources are present (oracle/ref/Makefile).
 *
 * Runs the reference's own host-side C code for the force step (the CPU
 * branches of BO_C, Atom_Energy_C -> Merge_Bonds_Atom_Energy_C_New,
 * Hydrogen_Bonds_C, Merge_Torsion_Valence_Angles,
 * vdW_Coulomb_Energy_Full_C_test_err, Add_All_dBond_to_Forces_C and the
 * H-bond list builder Init_Forces_noQEq_HB_Full_C) on the ghost atoms, far
 * list and uncorrected bond list the oracle builds, so that the oracle's
 * restatement of those routines is checked against the reference itself.
 *
 * The reference's own structures (reaxc_ctypes_sunway.h) are filled here;
 * this file includes the oracle's source to reach its internal lists.
 */
#include "../reax_oracle.c"

#undef SQR
#undef CUBE
#undef DEG2RAD
#undef constPI
#undef C_ele
#undef KCALpMOL_to_EV
#undef EV_TO_KCAL_PER_MOL
#undef HB_THRESHOLD
#undef MIN_SINE
#include "reaxc_defs_sunway.h"
#include "reaxc_ctypes_sunway.h"

/* the reference entry points (their pack structs all start with the
 * fields of ref_pack; only those are read by the CPU branches) */
typedef struct {
  reax_system_c *system;
  control_params *control;
  simulation_data *data;
  storage *workspace;
  reax_list **lists;
  output_controls *out_control;
  MPI_Comm comm;
  char tail[16384];
} ref_pack;

void BO_C(void *);
void Atom_Energy_C(void *);
void Hydrogen_Bonds_C(void *);
void Merge_Torsion_Valence_Angles(void *);
void vdW_Coulomb_Energy_Full_C_test_err(void *);
void Init_Forces_noQEq_HB_Full_C(void *);
void Add_All_dBond_to_Forces_C(reax_system_c *, control_params *, simulation_data *,
                               storage *, reax_list **, mpi_datatypes *);

/* unresolved by the reference's C files (defined in its C++ layer):
 * Calculate_Theta / Calculate_dCos_Theta restated from
 * reaxc_valence_angles_sunway.cpp:49-79 */
void Calculate_Theta(rvec dvec_ji, double d_ji, rvec dvec_jk, double d_jk, double *theta,
                     double *cos_theta) {
  calc_theta(dvec_ji, d_ji, dvec_jk, d_jk, theta, cos_theta);
}
void Calculate_dCos_Theta(rvec dvec_ji, double d_ji, rvec dvec_jk, double d_jk,
                          rvec *di, rvec *dj, rvec *dk) {
  calc_dcos_theta(dvec_ji, d_ji, dvec_jk, d_jk, *di, *dj, *dk);
}

static int ref_abort_code = 0;
void ro_stub_abort(int code) { ref_abort_code = code; }

static void *zalloc(size_t n) { return calloc(n ? n : 1, 1); }

/* Reference force step on the oracle's lists.  f_out[3n], energies as
 * ro_compute (pvector order + eng_vdwl, eng_coul, physical e_pol), bo_out
 * (optional) = corrected BO of every local-atom bond entry, in the oracle's
 * bond order. */
int ro_ref_compute(ro_ctx *c, double *f_out, double *energies, double *bo_out,
                   int *hb_ti, int *hb_tj, int *hb_img, long long *n_hb) {
  int i, k, t1, t2, t3, t4;
  const ffield_t *ff = &c->ff;
  const int nt = ff->ntypes;
  prepare_lists(c);
  build_bonds(c);
  const int N = c->N, n = c->n;

  /* force field in the reference layout */
  reax_interaction R;
  memset(&R, 0, sizeof R);
  R.num_atom_types = nt;
  R.gp.n_global = ff->ngp;
  R.gp.l = (double *)ff->gp;
  R.gp.vdw_type = ff->vdw_type;
  R.sbp = (single_body_parameters *)zalloc(nt * sizeof(single_body_parameters));
  for (t1 = 0; t1 < nt; t1++) {
    const sbp_t *s = &ff->sbp[t1];
    single_body_parameters *r = &R.sbp[t1];
    strncpy(r->name, s->name, 14);
    r->r_s = s->r_s; r->valency = s->valency; r->mass = s->mass; r->r_vdw = s->r_vdw;
    r->epsilon = s->epsilon; r->gamma = s->gamma; r->r_pi = s->r_pi;
    r->valency_e = s->valency_e; r->nlp_opt = s->nlp_opt; r->alpha = s->alpha;
    r->gamma_w = s->gamma_w; r->valency_boc = s->valency_boc; r->p_ovun5 = s->p_ovun5;
    r->chi = s->chi; r->eta = s->eta; r->p_hbond = s->p_hbond; r->r_pi_pi = s->r_pi_pi;
    r->p_lp2 = s->p_lp2; r->b_o_131 = s->b_o_131; r->b_o_132 = s->b_o_132;
    r->b_o_133 = s->b_o_133; r->p_ovun2 = s->p_ovun2; r->p_val3 = s->p_val3;
    r->valency_val = s->valency_val; r->p_val5 = s->p_val5; r->rcore2 = s->rcore2;
    r->ecore2 = s->ecore2; r->acore2 = s->acore2; r->lgcij = s->lgcij; r->lgre = s->lgre;
  }
  R.tbp = (two_body_parameters **)zalloc(nt * sizeof(void *));
  R.thbp = (three_body_header ***)zalloc(nt * sizeof(void *));
  R.hbp = (hbond_parameters ***)zalloc(nt * sizeof(void *));
  R.fbp = (four_body_header ****)zalloc(nt * sizeof(void *));
  for (t1 = 0; t1 < nt; t1++) {
    R.tbp[t1] = (two_body_parameters *)zalloc(nt * sizeof(two_body_parameters));
    R.thbp[t1] = (three_body_header **)zalloc(nt * sizeof(void *));
    R.hbp[t1] = (hbond_parameters **)zalloc(nt * sizeof(void *));
    R.fbp[t1] = (four_body_header ***)zalloc(nt * sizeof(void *));
    for (t2 = 0; t2 < nt; t2++) {
      const tbp_t *s = &ff->tbp[t1][t2];
      two_body_parameters *r = &R.tbp[t1][t2];
      r->p_bo1 = s->p_bo1; r->p_bo2 = s->p_bo2; r->p_bo3 = s->p_bo3; r->p_bo4 = s->p_bo4;
      r->p_bo5 = s->p_bo5; r->p_bo6 = s->p_bo6; r->r_s = s->r_s; r->r_p = s->r_p;
      r->r_pp = s->r_pp; r->p_boc3 = s->p_boc3; r->p_boc4 = s->p_boc4; r->p_boc5 = s->p_boc5;
      r->p_be1 = s->p_be1; r->p_be2 = s->p_be2; r->De_s = s->De_s; r->De_p = s->De_p;
      r->De_pp = s->De_pp; r->p_ovun1 = s->p_ovun1; r->D = s->D; r->alpha = s->alpha;
      r->r_vdW = s->r_vdW; r->gamma_w = s->gamma_w; r->rcore = s->rcore; r->ecore = s->ecore;
      r->acore = s->acore; r->lgcij = s->lgcij; r->lgre = s->lgre; r->gamma = s->gamma;
      r->v13cor = s->v13cor; r->ovc = s->ovc;
      R.thbp[t1][t2] = (three_body_header *)zalloc(nt * sizeof(three_body_header));
      R.hbp[t1][t2] = (hbond_parameters *)zalloc(nt * sizeof(hbond_parameters));
      R.fbp[t1][t2] = (four_body_header **)zalloc(nt * sizeof(void *));
      for (t3 = 0; t3 < nt; t3++) {
        const thbh_t *s3 = &ff->thbp[t1][t2][t3];
        three_body_header *r3 = &R.thbp[t1][t2][t3];
        r3->cnt = s3->cnt;
        for (k = 0; k < s3->cnt && k < REAX_MAX_3BODY_PARAM; k++) {
          r3->prm[k].theta_00 = s3->prm[k].theta_00; r3->prm[k].p_val1 = s3->prm[k].p_val1;
          r3->prm[k].p_val2 = s3->prm[k].p_val2; r3->prm[k].p_val4 = s3->prm[k].p_val4;
          r3->prm[k].p_val7 = s3->prm[k].p_val7; r3->prm[k].p_pen1 = s3->prm[k].p_pen1;
          r3->prm[k].p_coa1 = s3->prm[k].p_coa1;
        }
        R.hbp[t1][t2][t3].r0_hb = ff->hbp[t1][t2][t3].r0_hb;
        R.hbp[t1][t2][t3].p_hb1 = ff->hbp[t1][t2][t3].p_hb1;
        R.hbp[t1][t2][t3].p_hb2 = ff->hbp[t1][t2][t3].p_hb2;
        R.hbp[t1][t2][t3].p_hb3 = ff->hbp[t1][t2][t3].p_hb3;
        R.fbp[t1][t2][t3] = (four_body_header *)zalloc(nt * sizeof(four_body_header));
        for (t4 = 0; t4 < nt; t4++) {
          const fbh_t *s4 = &ff->fbp[t1][t2][t3][t4];
          four_body_header *r4 = &R.fbp[t1][t2][t3][t4];
          r4->cnt = s4->cnt;
          r4->prm[0].V1 = s4->prm.V1; r4->prm[0].V2 = s4->prm.V2; r4->prm[0].V3 = s4->prm.V3;
          r4->prm[0].p_tor1 = s4->prm.p_tor1; r4->prm[0].p_cot1 = s4->prm.p_cot1;
        }
      }
    }
  }

  /* system */
  reax_system_c *sys = (reax_system_c *)zalloc(sizeof(reax_system_c));
  sys->reax_param = R;
  sys->n = n;
  sys->N = N;
  sys->bigN = n;
  sys->packed_atoms = (atom_pack_t *)zalloc(N * sizeof(atom_pack_t));
  sys->Hindex = (int *)zalloc(N * sizeof(int));
  sys->num_bonds = (int *)zalloc(N * sizeof(int));
  sys->num_hbonds = (int *)zalloc(N * sizeof(int));
  int numH = 0;
  for (i = 0; i < N; i++) {
    atom_pack_t *a = &sys->packed_atoms[i];
    a->orig_id = c->tag[c->own[i]];
    a->type = c->te[i];
    a->x[0] = c->xe[3 * i]; a->x[1] = c->xe[3 * i + 1]; a->x[2] = c->xe[3 * i + 2];
    a->q = c->q[c->own[i]];
    if (i < n && ff->sbp[c->te[i]].p_hbond == 1) sys->Hindex[i] = numH++;
    else sys->Hindex[i] = -1;
  }
  sys->numH = numH;
  sys->evflag = 1;
  sys->eflag_global = 1;
  sys->vflag_global = 0;
  /* per-atom tallies (LAMMPS eflag_atom / vflag_atom) */
  sys->eflag_atom = 1;
  sys->vflag_atom = 1;
  sys->eatom = (double *)zalloc(N * sizeof(double));
  sys->vatom = (double (*)[6])zalloc(N * 6 * sizeof(double));
  sys->saferzone = 1.4;

  control_params *ctl = (control_params *)zalloc(sizeof(control_params));
  ctl->bo_cut = c->bo_cut;
  ctl->bond_cut = c->ctl.bond_cut;
  ctl->hbond_cut = c->ctl.hbond_cut;
  ctl->nonb_cut = c->nonb_cut;
  ctl->nonb_low = c->nonb_low;
  ctl->thb_cut = c->ctl.thb_cut;
  ctl->thb_cutsq = c->ctl.thb_cutsq;
  ctl->virial = 0;
  ctl->lgflag = c->ctl.lgflag;
  ctl->enobondsflag = c->ctl.enobondsflag;
  ctl->reneighbor = 1;
  simulation_data *data = (simulation_data *)zalloc(sizeof(simulation_data));
  output_controls *outc = (output_controls *)zalloc(sizeof(output_controls));
  mpi_datatypes *mpid = (mpi_datatypes *)zalloc(sizeof(mpi_datatypes));

  storage *ws = (storage *)zalloc(sizeof(storage));
  ws->bo_dboc = (rvec2 *)zalloc(N * sizeof(rvec2));
#define WS(f) ws->f = (double *)zalloc(N * sizeof(double))
  WS(Deltap); WS(Deltap_boc); WS(Delta); WS(Delta_lp); WS(Delta_lp_temp); WS(Delta_e);
  WS(Delta_val); WS(dDelta_lp); WS(dDelta_lp_temp); WS(nlp); WS(nlp_temp); WS(Clp); WS(vlpex);
#undef WS
  ws->dDeltap_self = (rvec *)zalloc(N * sizeof(rvec));
  ws->bond_mark = (int *)zalloc(N * sizeof(int));
  ws->fCdDelta = (rvec4 *)zalloc(N * sizeof(rvec4));
  for (k = 0; k < 8; k++) ws->Tap[k] = c->Tap[k];
  for (i = 0; i < N; i++) {
    ws->bo_dboc[i][0] = c->bo_dboc0[i];
    ws->dDeltap_self[i][0] = c->dDeltap_self[3 * i];
    ws->dDeltap_self[i][1] = c->dDeltap_self[3 * i + 1];
    ws->dDeltap_self[i][2] = c->dDeltap_self[3 * i + 2];
  }

  /* lists */
  reax_list *lists = (reax_list *)zalloc(LIST_N * sizeof(reax_list));
  reax_list *far = lists + FAR_NBRS_FULL, *bonds = lists + BONDS, *hb = lists + HBONDS;
  const long long nfar = c->far_start[N];
  far->n = N;
  far->num_intrs = (int)nfar;
  far->index = (int *)zalloc(N * sizeof(int));
  far->end_index = (int *)zalloc(N * sizeof(int));
  far->select.far_nbr_list_full =
      (far_neighbor_data_full *)zalloc(nfar * sizeof(far_neighbor_data_full));
  for (i = 0; i < N; i++) {
    far->index[i] = c->far_start[i];
    far->end_index[i] = c->far_start[i + 1];
  }
  for (long long p = 0; p < nfar; p++) {
    far_neighbor_data_full *e = &far->select.far_nbr_list_full[p];
    int j = c->far_nbr[p];
    e->nbr = j;
    e->type = c->te[j];
    e->orig_id = c->tag[c->own[j]];
    e->d = c->far_d[p];
    e->q = c->q[c->own[j]];
    e->dvec[0] = c->far_dvec[3 * p];
    e->dvec[1] = c->far_dvec[3 * p + 1];
    e->dvec[2] = c->far_dvec[3 * p + 2];
  }
  long long nb = 0;
  for (i = 0; i < N; i++) nb += c->b_end[i] - c->b_start[i];
  const long long bcap = c->b_end[N - 1] + 1;
  bonds->n = N;
  bonds->num_intrs = (int)bcap;
  bonds->index = (int *)zalloc(N * sizeof(int));
  bonds->end_index = (int *)zalloc(N * sizeof(int));
  bonds->select.bond_list = (bond_data *)zalloc(bcap * sizeof(bond_data));
  bonds->bo_data_list = (bond_order_data *)zalloc(bcap * sizeof(bond_order_data));
  bonds->BO_list = (double *)zalloc(bcap * sizeof(double));
  bonds->BOpi_list = (rvec2 *)zalloc(bcap * sizeof(rvec2));
  bonds->Cdbo_list = (double *)zalloc(bcap * sizeof(double));
  bonds->Cdbopi_list = (double *)zalloc(bcap * sizeof(double));
  bonds->Cdbopi2_list = (double *)zalloc(bcap * sizeof(double));
  for (i = 0; i < N; i++) {
    bonds->index[i] = c->b_start[i];
    bonds->end_index[i] = c->b_end[i];
    int p;
    for (p = c->b_start[i]; p < c->b_end[i]; p++) {
      const bond_t *b = &c->bonds[p];
      bond_data *r = &bonds->select.bond_list[p];
      bond_order_data *o = &bonds->bo_data_list[p];
      r->d = b->d;
      r->dvec[0] = b->dvec[0]; r->dvec[1] = b->dvec[1]; r->dvec[2] = b->dvec[2];
      r->nbr = b->nbr;
      r->dbond_index = p;
      r->sym_index = -1;   /* found by BO_Section2_C */
      bonds->BO_list[p] = b->BO;
      bonds->BOpi_list[p][0] = b->BO_pi;
      bonds->BOpi_list[p][1] = b->BO_pi2;
      o->BO_s = b->BO_s;
      for (k = 0; k < 3; k++) {
        o->dBOp[k] = b->dBOp[k];
        o->dln_BOp_s[k] = b->dln_BOp_s[k];
        o->dln_BOp_pi[k] = b->dln_BOp_pi[k];
        o->dln_BOp_pi2[k] = b->dln_BOp_pi2[k];
      }
    }
  }
  /* H-bond list: built by the reference's own Init_Forces_noQEq_HB_Full_C
   * from the far list; slots sized from the oracle's far-list rows */
  hb->n = numH;
  hb->index = (int *)zalloc((numH + 1) * sizeof(int));
  hb->end_index = (int *)zalloc((numH + 1) * sizeof(int));
  long long hcap = 0;
  for (i = 0; i < n; i++)
    if (sys->Hindex[i] >= 0) {
      hb->index[sys->Hindex[i]] = (int)hcap;
      hb->end_index[sys->Hindex[i]] = (int)hcap;
      hcap += c->far_start[i + 1] - c->far_start[i];
    }
  hb->num_intrs = (int)hcap;
  hb->select.hbond_list = (hbond_data *)zalloc((hcap + 1) * sizeof(hbond_data));

  ref_pack pk;
  memset(&pk, 0, sizeof pk);
  pk.system = sys;
  pk.control = ctl;
  pk.data = data;
  pk.workspace = ws;
  pk.lists = &lists;
  pk.out_control = outc;
  ref_abort_code = 0;
  Init_Forces_noQEq_HB_Full_C(&pk);
  vdW_Coulomb_Energy_Full_C_test_err(&pk);
  BO_C(&pk);
  Atom_Energy_C(&pk);
  Hydrogen_Bonds_C(&pk);
  Merge_Torsion_Valence_Angles(&pk);
  Add_All_dBond_to_Forces_C(sys, ctl, data, ws, &lists, mpid);

  /* results */
  tally_alloc(c);
  for (i = 0; i < n; i++) {
    c->ref_eatom[i] = sys->eatom[i];
    for (k = 0; k < 6; k++) c->ref_vatom[6 * i + k] = sys->vatom[i][k];
  }
  for (i = 0; i < 3 * n; i++) f_out[i] = 0.0;
  for (i = 0; i < N; i++) {
    int o = c->own[i];
    f_out[3 * o + 0] -= ws->fCdDelta[i][0];
    f_out[3 * o + 1] -= ws->fCdDelta[i][1];
    f_out[3 * o + 2] -= ws->fCdDelta[i][2];
  }
  energy_data *e = &data->my_en;
  double en[RO_NENERGY] = {0};
  en[RO_E_BOND] = e->e_bond;
  en[RO_E_OVUN] = e->e_ov + e->e_un;
  en[RO_E_LP] = e->e_lp;
  en[RO_E_ANG] = e->e_ang;
  en[RO_E_PEN] = e->e_pen;
  en[RO_E_COA] = e->e_coa;
  en[RO_E_HB] = e->e_hb;
  en[RO_E_TOR] = e->e_tor;
  en[RO_E_CON] = e->e_con;
  en[RO_E_VDW] = e->e_vdW;
  en[RO_E_ELE] = e->e_ele;
  en[RO_E_POL] = e->e_pol;
  en[RO_ENG_VDWL] = sys->eng_vdwl;
  en[RO_ENG_COUL] = sys->eng_coul;
  en[RO_E_POL_PHYS] = 0.0;
  if (energies) memcpy(energies, en, sizeof en);
  if (bo_out) {
    long long q = 0;
    int p;
    for (i = 0; i < n; i++)
      for (p = c->b_start[i]; p < c->b_end[i]; p++, q++) {
        bo_out[4 * q + 0] = bonds->BO_list[p];
        bo_out[4 * q + 1] = bonds->bo_data_list[p].BO_s;
        bo_out[4 * q + 2] = bonds->BOpi_list[p][0];
        bo_out[4 * q + 3] = bonds->BOpi_list[p][1];
      }
  }
  /* the reference's H-bond list as (tag_i, tag_j, image of j) */
  long long nhb_ref = 0;
  for (i = 0; i < n; i++) {
    if (sys->Hindex[i] < 0) continue;
    int p;
    for (p = hb->index[sys->Hindex[i]]; p < hb->end_index[sys->Hindex[i]]; p++, nhb_ref++) {
      if (!hb_ti) continue;
      int j = hb->select.hbond_list[p].nbr;
      hb_ti[nhb_ref] = c->tag[i];
      hb_tj[nhb_ref] = c->tag[c->own[j]];
      hb_img[nhb_ref] = c->imgc[j];
    }
  }
  if (n_hb) *n_hb = nhb_ref;

  /* free */
  for (t1 = 0; t1 < nt; t1++) {
    for (t2 = 0; t2 < nt; t2++) {
      for (t3 = 0; t3 < nt; t3++) free(R.fbp[t1][t2][t3]);
      free(R.thbp[t1][t2]); free(R.hbp[t1][t2]); free(R.fbp[t1][t2]);
    }
    free(R.tbp[t1]); free(R.thbp[t1]); free(R.hbp[t1]); free(R.fbp[t1]);
  }
  free(R.sbp); free(R.tbp); free(R.thbp); free(R.hbp); free(R.fbp);
  free(sys->packed_atoms); free(sys->eatom); free(sys->vatom); free(sys->Hindex); free(sys->num_bonds); free(sys->num_hbonds);
  free(sys); free(ctl); free(data); free(outc); free(mpid);
  free(ws->bo_dboc); free(ws->Deltap); free(ws->Deltap_boc); free(ws->Delta);
  free(ws->Delta_lp); free(ws->Delta_lp_temp); free(ws->Delta_e); free(ws->Delta_val);
  free(ws->dDelta_lp); free(ws->dDelta_lp_temp); free(ws->nlp); free(ws->nlp_temp);
  free(ws->Clp); free(ws->vlpex); free(ws->dDeltap_self); free(ws->bond_mark);
  free(ws->fCdDelta); free(ws);
  free(far->index); free(far->end_index); free(far->select.far_nbr_list_full);
  free(bonds->index); free(bonds->end_index); free(bonds->select.bond_list);
  free(bonds->bo_data_list); free(bonds->BO_list); free(bonds->BOpi_list);
  free(bonds->Cdbo_list); free(bonds->Cdbopi_list); free(bonds->Cdbopi2_list);
  free(hb->index); free(hb->end_index); free(hb->select.hbond_list);
  free(lists);
  return ref_abort_code;
}

/* ------------------------------------------------------------------ */
/* QEq through the reference's own FixQEqReaxSunway::pre_force
 * (ref_qeq.cpp) on the oracle's H matrix */

int ref_qeq_pre_force(int n, const int *type, int ntypes, const double *chi,
                      const double *eta, const int *start, const int *col,
                      const double *val, double tol, double *s_hist, double *t_hist,
                      double *s, double *t, double *q_out, int *iters_s, int *iters_t);

static int ref_qeq_driver(ro_ctx *c, const void *Hv, int *iters_s, int *iters_t) {
  const hmat_t *H = (const hmat_t *)Hv;
  const int nt = c->ff.ntypes;
  double *chi = (double *)malloc(nt * sizeof(double));
  double *eta = (double *)malloc(nt * sizeof(double));
  int k, warn;
  for (k = 0; k < nt; k++) {
    chi[k] = c->ff.sbp[k].chi;
    eta[k] = c->ff.sbp[k].eta;
  }
  warn = ref_qeq_pre_force(c->n, c->type, nt, chi, eta, H->start, H->col, H->val,
                           c->ctl.qeq_tol, c->s_hist, c->t_hist, c->s, c->t, c->q,
                           iters_s, iters_t);
  free(chi);
  free(eta);
  return warn ? 1 : 0;
}

/* on != 0: this context's ro_qeq (and ro_run_nve's QEq) run the
 * reference's pre_force; 0: the oracle's restatement */
void ro_ref_use_qeq(ro_ctx *c, int on) { c->qeq_driver = on ? ref_qeq_driver : NULL; }

/* the reference's per-atom tallies (eatom[n], vatom[6n]) of the last
 * ro_ref_compute */
void ro_ref_atom_tallies(const ro_ctx *c, double *eatom, double *vatom) {
  if (c->tally_n != c->n) return;
  if (eatom) memcpy(eatom, c->ref_eatom, (size_t)c->n * sizeof(double));
  if (vatom) memcpy(vatom, c->ref_vatom, 6 * (size_t)c->n * sizeof(double));
}
