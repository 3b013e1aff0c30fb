// Cell binning, atom sort, pair list, bond list and H-bond partner list.
//
// Replaces, on the GPU:
//  * the binned full/ghost neighbour build (npair_full_bin_atomonly_sw5.c:
//    57-181, npair_full_bin_ghost_sw5.c:80-231) and the far-list filter to
//    d <= nonb_cut (write_reax_lists_c, pair_reaxc_sw64.c:42-96);
//  * the QEq H-matrix build (compute_H_Full_C, fix_qeq_reax_sw64.c:768-911),
//    fused into the pair-list pass because it uses the same pairs;
//  * the uncorrected bond orders and the full bond list
//    (Init_Forces_noQEq_Full_C_para, reaxc_forces_sw64.c:996-1318; CPU form
//    BOp_single, reaxc_forces_sunway.cpp:677-825);
//  * the H-bond partner list (Init_Forces_noQEq_HB_Full_C,
//    reaxc_forces_sw64.c:787-863).
//
// Instead of ghost atoms every atom is local and each list entry carries the
// periodic image of its partner.  Membership tests (d^2 <= cut^2, d <=
// bond_cut, BO' >= bo_cut, d <= hbond_cut) are evaluated in FP64 with
// explicitly rounded, non-contracted operations so that they reproduce the
// reference's decisions bit for bit.
#include <cstdio>

#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// wrap into [0,L) like the host oracle: x - L*floor(x/L), rounded per op
__device__ __forceinline__ double wrap1(double x, double L) {
  double y = __dsub_rn(x, __dmul_rn(L, floor(__ddiv_rn(x, L))));
  if (y >= L) y = __dsub_rn(y, L);
  if (y < 0.0) y = 0.0;
  return y;
}

__device__ __forceinline__ int cell_of(double x, double w, int nc) {
  int c = (int)(x / w);
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

__device__ __forceinline__ int frac_cell(double u, int nc) {
  int c = (int)floor(u * nc);
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// cell of a wrapped position: Cartesian cells of an orthogonal segment,
// cells of the fractional coordinates of a triclinic one
__device__ __forceinline__ void cell3(const SegGeom &g, double x, double y, double z, int &cx,
                                      int &cy, int &cz) {
  if (!g.tri) {
    cx = cell_of(x, g.cellw[0], g.nc[0]);
    cy = cell_of(y, g.cellw[1], g.nc[1]);
    cz = cell_of(z, g.cellw[2], g.nc[2]);
  } else {
    double u, v, w;
    frac3(g, x, y, z, u, v, w);
    cx = frac_cell(u, g.nc[0]);
    cy = frac_cell(v, g.nc[1]);
    cz = frac_cell(w, g.nc[2]);
  }
}

// triclinic wrap: subtract the lattice translation floor(fractional
// coordinates), rounded per operation like the oracle
__device__ __forceinline__ void wrap_tri(const SegGeom &g, double &x, double &y, double &z) {
  double u, v, w;
  frac3(g, x, y, z, u, v, w);
  const double kx = floor(u), ky = floor(v), kz = floor(w);
  x = __dsub_rn(x, __dadd_rn(__dadd_rn(__dmul_rn(kx, g.L[0]), __dmul_rn(ky, g.tilt[0])),
                             __dmul_rn(kz, g.tilt[1])));
  y = __dsub_rn(y, __dadd_rn(__dmul_rn(ky, g.L[1]), __dmul_rn(kz, g.tilt[2])));
  z = __dsub_rn(z, __dmul_rn(kz, g.L[2]));
}

// -------------------------------------------------------------------
// binning and sort

__global__ void k_cell_assign(Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const SegGeom &g = d.seg[d.seg_o[i]];
  double x = d.x_o[3 * i + 0], y = d.x_o[3 * i + 1], z = d.x_o[3 * i + 2];
  if (!g.tri) {
    x = wrap1(x, g.L[0]);
    y = wrap1(y, g.L[1]);
    z = wrap1(z, g.L[2]);
  } else {
    wrap_tri(g, x, y, z);
  }
  d.x_o[3 * i + 0] = x;
  d.x_o[3 * i + 1] = y;
  d.x_o[3 * i + 2] = z;
  int cx, cy, cz;
  cell3(g, x, y, z, cx, cy, cz);
  int c = g.cell0 + (cz * g.nc[1] + cy) * g.nc[0] + cx;
  d.cell_o[i] = c;
  atomicAdd(&d.cell_count[c], 1);
}

// exclusive scan of cell_count into cell_start (one block per 1024 cells,
// then a single-block pass over block sums; enough for < 1M cells)
__global__ void k_scan_blocks(const int *in, int *out, int *bsum, int n) {
  __shared__ int s[1024];
  int t = threadIdx.x, g = blockIdx.x * 1024 + t;
  int v = g < n ? in[g] : 0;
  s[t] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int a = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += a;
    __syncthreads();
  }
  if (g < n) out[g] = s[t] - v;
  if (t == 1023) bsum[blockIdx.x] = s[t];
}

__global__ void k_scan_sums(int *bsum, int nb, int *total_out) {
  __shared__ int s[1024];
  int t = threadIdx.x;
  // serial over chunks of 1024
  int carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    int v = base + t < nb ? bsum[base + t] : 0;
    s[t] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      int a = t >= off ? s[t - off] : 0;
      __syncthreads();
      s[t] += a;
      __syncthreads();
    }
    if (base + t < nb) bsum[base + t] = carry + s[t] - v;
    int tot = s[1023];
    __syncthreads();
    carry += tot;
  }
  if (t == 0 && total_out) *total_out = carry;
}

__global__ void k_scan_add(int *out, const int *bsum, int n) {
  int g = blockIdx.x * 1024 + threadIdx.x;
  if (g < n) out[g] += bsum[blockIdx.x];
}

__global__ void k_scatter(Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  int c = d.cell_o[i];
  int slot = d.cell_start[c] + atomicAdd(&d.cell_fill[c], 1);
  d.perm[slot] = i;
}

// deterministic order inside a cell: by original index
__global__ void k_cell_order(Dev d, int ncell) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  int b = d.cell_start[c], e = d.cell_start[c + 1];
  for (int a = b + 1; a < e; ++a) {
    int v = d.perm[a], z = a - 1;
    while (z >= b && d.perm[z] > v) {
      d.perm[z + 1] = d.perm[z];
      --z;
    }
    d.perm[z + 1] = v;
  }
}

__global__ void k_gather(Dev d) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  int i = d.perm[s];
  double x = d.x_o[3 * i], y = d.x_o[3 * i + 1], z = d.x_o[3 * i + 2];
  d.xs[s] = make_double4(x, y, z, d.q_o[i]);
  int t = d.type_o[i];
  const float hx = __double2float_rn(x), hy = __double2float_rn(y), hz = __double2float_rn(z);
  d.xf[s] = make_float4(hx, hy, hz, __int_as_float(t));
  const double q = d.q_o[i];
  const float qh = __double2float_rn(q);
  d.xl[s] = make_float4(__double2float_rn(x - (double)hx), __double2float_rn(y - (double)hy),
                        __double2float_rn(z - (double)hz), qh);
  d.qlo[s] = __double2float_rn(q - (double)qh);
  d.ts[s] = t;
  d.tags[s] = d.tag_o[i];
  d.seg_s[s] = d.seg_o[i];
  d.iperm[i] = s;
}

// -------------------------------------------------------------------
// pair list (full, both directions) + QEq H values
//
// One warp per atom i walks the half of the cell stencil at
// lexicographically non-negative offsets (oz, oy, ox) >= (0, 0, 0), taking
// in its own cell (offset 0, image 0) only partners j > i: every unordered
// pair (i, j, image) is found once, by one warp, which evaluates the H_ij
// value once and writes both directed entries -- (j, image) into row i and
// (i, -image) into row j.  A row's near and far parts are filled by atomic
// claims (one per warp batch for row i, one per entry for the partner
// rows), so the order inside a part depends on scheduling; every consumer
// sums or filters a row's entries without regard to their order.
//
// The walk goes along x in runs of consecutive cells (contiguous ranges of
// the cell-sorted atoms), 32 candidates per step (FP32 distance prefilter
// with a safety margin); survivors go to a per-warp shared queue, and every
// full batch of 32 is finished with all lanes busy: list membership and the
// near/far split of each direction (from the FP32 (hi, lo) distance, or the
// exact FP64 distance of that direction within 1e-5 of a cutoff, so each
// directed entry is decided exactly as the oracle decides it), and H.

constexpr int NB_WARPS = 8;          // warps per block in k_build_nbrs
constexpr int QCAP = 64;             // queue slots per warp

struct NbrQueue {
  int j[QCAP];
  int img[QCAP];
};

// exact (FP64, explicitly rounded) squared distance from an atom at xi to
// the image (sx, sy, sz) of sorted atom j
__device__ __forceinline__ double exact_d2(const Dev &d, int j, int sx, int sy, int sz,
                                          const double4 &xi, const SegGeom &g) {
  double dx, dy, dz;
  disp64(g, d.xs[j], xi, sx, sy, sz, dx, dy, dz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// the reference's near membership, d <= near_cut, from an exact d^2
__device__ __forceinline__ bool near_exact(double e2, const Control &C) {
  if (e2 <= C.near_cut2_lo) return true;
  if (e2 > C.near_cut2_hi) return false;
  return __dsqrt_rn(e2) <= C.near_cut;
}

// FP32 tests are taken only when d^2 is more than this relative distance
// from the cutoff; the FP32 d^2 from df_disp is good to a few 1e-7, so the
// outcome is the FP64 one
constexpr float MARGIN32 = 1e-5f;

// QEq H_ij of a listed pair from its r^2: the mixed form in FP32 from the
// FP32 r^2 (h32), the FP64 form from the FMA-rounded FP64 r^2 (h), from the
// FP64 table or analytically
template <bool MIXED>
__device__ __forceinline__ void pair_h(const Dev &d, const Control &C, const ForceField &F,
                                       int ti, int tj, double d2, float d2f, double &h,
                                       float &h32) {
  h = 0.0;
  h32 = 0.f;
  if (MIXED) {
    if (d2f <= C.swb2_f) {
      // FP32: factored taper when swa = 0
      const float r = d2f * rsqrtf(d2f);
      float tp;
      if (C.qtap_factored) {
        const float t = r * C.inv_swb_q_f, u = 1.f - t, u2 = u * u;
        tp = u2 * u2 * (1.f + t * (4.f + t * (10.f + t * 20.f)));
      } else {
        const float *T = C.qTap_f;
        tp = fmaf(T[7], r, T[6]);
        tp = fmaf(tp, r, T[5]);
        tp = fmaf(tp, r, T[4]);
        tp = fmaf(tp, r, T[3]);
        tp = fmaf(tp, r, T[2]);
        tp = fmaf(tp, r, T[1]);
        tp = fmaf(tp, r, T[0]);
      }
      const float x = fmaf(d2f, r, C.nb32[ti][tj].gamma);
      h32 = tp * 14.4f * rcbrtf(x);
    }
  } else if (!(C.h_all_listed || d2 <= C.swb2)) {
    h = 0.0;
  } else if (C.tab_n && d2f >= C.tab_s0_f) {
    // FP64 table of H_ij (cubic Hermite in r^2, power basis per interval)
    const double x = fma(d2, C.tab_inv_ds, C.tab_x0);
    int k = (int)x;
    if (k > C.tab_n - 1) k = C.tab_n - 1;
    const double u = x - (double)k;
    const double2 *T =
        reinterpret_cast<const double2 *>(d.tab_h + ((long long)C.tab_pair[ti][tj] * C.tab_n + k) * 4);
    const double2 c01 = T[0], c23 = T[1];
    h = fma(fma(fma(c23.y, u, c23.x), u, c01.y), u, c01.x);
  } else {
    // H_ij = Tap(r) * 14.4 / (r^3 + shld)^c, c = 0.3333333333333
    const double r = d2 * rsqrt(d2);
    const double *T = C.qTap;
    double tp = fma(T[7], r, T[6]);
    tp = fma(tp, r, T[5]);
    tp = fma(tp, r, T[4]);
    tp = fma(tp, r, T[3]);
    tp = fma(tp, r, T[2]);
    tp = fma(tp, r, T[1]);
    tp = fma(tp, r, T[0]);
    const double x = fma(d2, r, F.tbp[ti][tj].gamma);
    h = tp * 14.4 * rpow_third(x, RG_C3_QEQ);
  }
}

// FP64 form, orthogonal segments: H_ij from the FP64 table with r^2, the
// interval offset and the cubic as FP32 pairs (~1e-13 relative, far below
// the table's 1e-10), on the FP32 units only
__device__ __forceinline__ fpair pair_h_fp(const Dev &d, const Control &C, int ti, int tj,
                                           fpair s2) {
  int k;
  fpair u;
  fp_interval(C, s2, k, u);
  const float4 *T = d.tab_h_fp + ((long long)C.tab_pair[ti][tj] * C.tab_n + k) * 2;
  return fp_cubic(T[0], T[1], u);
}

// an FP64 H_ij as the FP32 pair the FP64 form stores
__device__ __forceinline__ float2 h_pair(double h) {
  const float hi = __double2float_rn(h);
  return make_float2(hi, __double2float_rn(h - (double)hi));
}

// whether the FP64 form takes H_ij from pair_h_fp
__device__ __forceinline__ bool use_h_fp(const Dev &d, const Control &C, const SegGeom &g,
                                         float d2f) {
  return d.tab_h_fp && C.h_all_listed && !g.tri && d2f >= C.tab_s0_f;
}

template <bool MIXED>
__device__ __forceinline__ void nbr_flush(const Dev &d, const Control &C, const ForceField &F,
                                          const NbrQueue &Q, int cnt, int lane, int i,
                                          const double4 &xi, const float4 &xif, const float4 &xil,
                                          int ti, const SegGeom &g) {
  bool in = false, near = false, in_m = false, near_m = false, hfp = false;
  double d2 = 0.0;
  float d2f = 0.f;
  int j = 0, img = 0, sx = 0, sy = 0, sz = 0;
  float4 hj = make_float4(0.f, 0.f, 0.f, 0.f), lj = hj;
  if (lane < cnt) {
    j = Q.j[lane];
    img = Q.img[lane];
    img_unpack(img, &sx, &sy, &sz);
    hj = d.xf[j];
    lj = d.xl[j];
    float dx, dy, dz;
    disp32(g, hj, lj, xif, xil, sx, sy, sz, dx, dy, dz);
    d2f = dx * dx + dy * dy + dz * dz;
    const float lc2 = C.list_cut2_f;
    if (d2f <= lc2 * (1.f - MARGIN32)) {
      in = in_m = true;
    } else if (d2f <= lc2 * (1.f + MARGIN32)) {
      in = exact_d2(d, j, sx, sy, sz, xi, g) <= C.list_cut2;
      in_m = exact_d2(d, i, -sx, -sy, -sz, d.xs[j], g) <= C.list_cut2;
    }
    const float nc2 = C.near_cut_f * C.near_cut_f;
    if (MIXED) {
      // near part: conservative (the bond pass tests its own cutoffs)
      near = near_m = d2f <= nc2 * (1.f + MARGIN32);
    } else if (in || in_m) {
      if (d2f <= nc2 * (1.f - MARGIN32)) {
        near = near_m = true;
      } else if (d2f <= nc2 * (1.f + MARGIN32)) {
        near = near_exact(exact_d2(d, j, sx, sy, sz, xi, g), C);
        near_m = near_exact(exact_d2(d, i, -sx, -sy, -sz, d.xs[j], g), C);
      }
    }
    if (!MIXED && (in || in_m)) {
      hfp = use_h_fp(d, C, g, d2f);
      if (!hfp) {
        // r^2 for H: FMA-rounded from the exact displacement (the pair
        // functions are smooth; membership is decided above)
        double ex, ey, ez;
        disp64(g, d.xs[j], xi, sx, sy, sz, ex, ey, ez);
        d2 = fma(ex, ex, fma(ey, ey, ez * ez));
      }
    }
  }
  // row i: claim the batch's near and far slots with one atomic each
  const unsigned mn = __ballot_sync(FULL, in && near);
  const unsigned mf = __ballot_sync(FULL, in && !near);
  int baseN = 0, baseF = 0;
  if (lane == 0) {
    if (mn) baseN = atomicAdd(&d.n_near[i], __popc(mn));
    if (mf) baseF = atomicAdd(&d.n_far[i], __popc(mf));
  }
  baseN = __shfl_sync(FULL, baseN, 0);
  baseF = __shfl_sync(FULL, baseF, 0);
  if (!(in || in_m)) return;
  const int capN = d.nb_capN, capF = d.nb_cap - d.nb_capN;
  const int tj = __float_as_int(d.xf[j].w);
  double h = 0.0;
  float h32 = 0.f;
  float2 hp = make_float2(0.f, 0.f);   // FP64 form: H_ij as an FP32 pair
  if (!MIXED && hfp) {
    const fpair v = pair_h_fp(d, C, ti, tj, fp_d2(g, hj, lj, xif, xil, sx, sy, sz));
    hp = make_float2(v.hi, v.lo);
  } else {
    pair_h<MIXED>(d, C, F, ti, tj, d2, d2f, h, h32);
    if (!MIXED) hp = h_pair(h);
  }
  if (in) {
    const int p = near ? baseN + __popc(mn & lanemask_lt()) : baseF + __popc(mf & lanemask_lt());
    if (p < (near ? capN : capF)) {
      const long long slot = (long long)i * d.nb_cap + (near ? p : capN + p);
      d.nbr[slot] = ((uint32_t)j << 8) | (uint32_t)img;
      if (MIXED) d.hval32[slot] = h32;
      else d.hvalp[slot] = hp;
    }
  }
  if (in_m) {
    const int p = atomicAdd(near_m ? &d.n_near[j] : &d.n_far[j], 1);
    if (p < (near_m ? capN : capF)) {
      const long long slot = (long long)j * d.nb_cap + (near_m ? p : capN + p);
      d.nbr[slot] = ((uint32_t)i << 8) | (uint32_t)img_pack(-sx, -sy, -sz);
      if (MIXED) d.hval32[slot] = h32;
      else d.hvalp[slot] = hp;
    }
  }
}

template <bool MIXED>
__global__ void __launch_bounds__(NB_WARPS * 32, 3) k_build_nbrs(Dev d) {
  __shared__ NbrQueue queues[NB_WARPS];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= d.n) return;
  NbrQueue &Q = queues[wib];
  const Control &C = *d.ctl;
  const ForceField &F = *d.ff;
  const double4 xi = d.xs[i];
  const float4 xif = d.xf[i];
  const float4 xil = d.xl[i];
  const int ti = d.ts[i];
  const float cut2f = C.list_pre2_f;
  const SegGeom &g = d.seg[d.seg_s[i]];
  const int ncx = g.nc[0], ncy = g.nc[1], ncz = g.nc[2], S = g.S;
  // the cell the binning put atom i in (integer decomposition, no FP64)
  const int cl = d.cell_o[d.perm[i]] - g.cell0;
  const int cx = cl % ncx, cy = (cl / ncx) % ncy, cz = cl / (ncx * ncy);
  const int nx = ncx;
  int qn = 0;
  // Orthogonal segments clip the stencil to the cutoff sphere: a row of
  // cells (fixed oy, oz) whose y-z slab is farther from atom i than the
  // cutoff is skipped, and along x only the cells the sphere reaches at the
  // row's y-z distance are walked (FP32 geometry with the prefilter's
  // margin; the unwrapped cell indices give the periodic images' places).
  const bool clip = !g.tri;
  const float wy = g.cellw_f[1], wz = g.cellw_f[2], iwx = 1.f / g.cellw_f[0];
  for (int oz = 0; oz <= S; ++oz) {
    int rz = cz + oz, sz = 0;
    while (rz >= ncz) { rz -= ncz; ++sz; }
    float dz2 = 0.f;
    if (clip) {
      const float lo = (cz + oz) * wz - xif.z, hi = lo + wz;
      const float dz = lo > 0.f ? lo : (hi < 0.f ? -hi : 0.f);
      dz2 = dz * dz;
      if (dz2 > cut2f) continue;
    }
    for (int oy = (oz == 0 ? 0 : -S); oy <= S; ++oy) {
      int ry = cy + oy, sy = 0;
      while (ry < 0) { ry += ncy; --sy; }
      while (ry >= ncy) { ry -= ncy; ++sy; }
      int ox_lo = (oz == 0 && oy == 0) ? 0 : -S, ox_hi = S;
      if (clip) {
        const float lo = (cy + oy) * wy - xif.y, hi = lo + wy;
        const float dy = lo > 0.f ? lo : (hi < 0.f ? -hi : 0.f);
        const float r2 = cut2f - dz2 - dy * dy;
        if (r2 < 0.f) continue;
        const float rx_ = sqrtf(r2);
        // cells whose x-range meets [x_i - rx_, x_i + rx_]
        ox_lo = max(ox_lo, (int)floorf((xif.x - rx_) * iwx) - cx);
        ox_hi = min(ox_hi, (int)floorf((xif.x + rx_) * iwx) - cx);
      }
      const int rowcell = g.cell0 + (rz * ncy + ry) * nx;
      // runs of consecutive cells with one x image each
      int ox = ox_lo;
      while (ox <= ox_hi) {
        int rx = cx + ox, sx = 0;
        while (rx < 0) { rx += nx; --sx; }
        while (rx >= nx) { rx -= nx; ++sx; }
        int len = 1;
        while (ox + len <= ox_hi && rx + len < nx) ++len;
        const int beg = d.cell_start[rowcell + rx];
        const int end = d.cell_start[rowcell + rx + len];
        ox += len;
        // orthogonal: (float)(s L) exactly (|s| <= 2 scales the rounded edge
        // exactly); triclinic: the FP32 translation
        float shxf, shyf, shzf;
        img_vec32(g, sx, sy, sz, shxf, shyf, shzf);
        // image 0 arises only at offset (0, 0, ox >= 0): there the partners
        // are the atoms after i (its own cell's later atoms, the next cells)
        const bool self_img = (sx == 0 && sy == 0 && sz == 0);
        const int img = img_pack(sx, sy, sz);
        for (int base = (self_img ? max(beg, i + 1) : beg); base < end; base += 32) {
          const int j = base + lane;
          bool cand = false;
          if (j < end) {
            const float4 xjf = d.xf[j];
            const float fx = xjf.x + shxf - xif.x;
            const float fy = xjf.y + shyf - xif.y;
            const float fz = xjf.z + shzf - xif.z;
            cand = fx * fx + fy * fy + fz * fz <= cut2f;
          }
          const unsigned mc = __ballot_sync(FULL, cand);
          if (cand) {
            const int slot = qn + __popc(mc & lanemask_lt());
            Q.j[slot] = j;
            Q.img[slot] = img;
          }
          qn += __popc(mc);
          __syncwarp();
          if (qn >= 32) {
            nbr_flush<MIXED>(d, C, F, Q, 32, lane, i, xi, xif, xil, ti, g);
            __syncwarp();
            // move the leftover (< 32) to the front of the queue
            const int left = qn - 32;
            int lj = 0, limg = 0;
            if (lane < left) {
              lj = Q.j[32 + lane];
              limg = Q.img[32 + lane];
            }
            __syncwarp();
            if (lane < left) {
              Q.j[lane] = lj;
              Q.img[lane] = limg;
            }
            qn = left;
            __syncwarp();
          }
        }
      }
    }
  }
  if (qn > 0) nbr_flush<MIXED>(d, C, F, Q, qn, lane, i, xi, xif, xil, ti, g);
}

// -------------------------------------------------------------------
// pair list + QEq H values, per-cell tiles (the alternative the autotuner
// may pick over the warp-per-atom walk above)
//
// One block per cell A.  Its atoms, then each run of neighbour cells of the
// same half stencil (chunks of TB atoms), are staged in shared memory, FP32
// (hi, lo) and FP64 positions; every (a, b) pair of the tile is prefiltered
// in FP32 from shared memory into a queue.  For the queued pairs the block
// decides list membership and the near/far split of each direction (exactly
// as the warp walk), counts each row's new entries with shared atomics,
// claims the rows' slots with one global atomic per row part and tile,
// evaluates H once per pair and writes both directed entries.  The per-atom
// stencil loop and its per-candidate global loads become one pass per cell.

constexpr int TILE_T = 128;   // threads per block
constexpr int TA = 64;        // A atoms per tile
constexpr int TB = 128;       // neighbour atoms per tile
constexpr int TQ = 1024;      // candidate pairs per queue pass

struct PairTile {
  double4 ax[TA], bx[TB];
  float4 af[TA], al[TA], bf[TB], bl[TB];
  double d2[TQ];                 // FP64 form: FMA-rounded r^2 of queued pairs
  float d2f[TQ];
  uint32_t q[TQ];                // queued pair (a << 16) | b
  unsigned short rk[TQ][2];      // entry's rank in a's row part, in b's
  unsigned char fl[TQ];          // 1 in, 2 near, 4 mirror in, 8 mirror near
  int cnt[2][TA + TB];           // per row part: new entries, then claimed base
  int nq;
};

__device__ __forceinline__ int seg_of_cell(const Dev &d, int c) {
  int lo = 0, hi = d.nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.seg[mid].cell0 <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ double exact_d2v(const double4 &xj, int sx, int sy, int sz,
                                           const double4 &xi, const SegGeom &g) {
  double dx, dy, dz;
  disp64(g, xj, xi, sx, sy, sz, dx, dy, dz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

template <bool MIXED>
__global__ void __launch_bounds__(TILE_T) k_build_nbrs_tiles(Dev d) {
  __shared__ PairTile T;
  const int c = blockIdx.x;
  const int a_beg = d.cell_start[c], a_end = d.cell_start[c + 1];
  if (a_beg >= a_end) return;
  const Control &C = *d.ctl;
  const ForceField &F = *d.ff;
  const SegGeom &g = d.seg[seg_of_cell(d, c)];
  const int ncx = g.nc[0], ncy = g.nc[1], ncz = g.nc[2], S = g.S;
  const int cl = c - g.cell0;
  const int cx = cl % ncx, cy = (cl / ncx) % ncy, cz = cl / (ncx * ncy);
  const float cut2f = C.list_pre2_f;
  const float lc2 = C.list_cut2_f, nc2 = C.near_cut_f * C.near_cut_f;
  const bool clip = !g.tri;
  const float wx = g.cellw_f[0], wy = g.cellw_f[1], wz = g.cellw_f[2];
  const int tid = threadIdx.x;
  const int capN = d.nb_capN, capF = d.nb_cap - d.nb_capN;
  for (int a0 = a_beg; a0 < a_end; a0 += TA) {
    const int na = min(TA, a_end - a0);
    __syncthreads();
    for (int k = tid; k < na; k += TILE_T) {
      T.ax[k] = d.xs[a0 + k];
      T.af[k] = d.xf[a0 + k];
      T.al[k] = d.xl[a0 + k];
    }
    for (int oz = 0; oz <= S; ++oz) {
      int rz = cz + oz, sz = 0;
      while (rz >= ncz) { rz -= ncz; ++sz; }
      // orthogonal: gaps between cell A's slab and the row's (FP32 with the
      // prefilter's margin)
      const float gz = clip ? (float)max(0, oz - 1) * wz : 0.f;
      if (gz * gz > cut2f) continue;
      for (int oy = (oz == 0 ? 0 : -S); oy <= S; ++oy) {
        int ry = cy + oy, sy = 0;
        while (ry < 0) { ry += ncy; --sy; }
        while (ry >= ncy) { ry -= ncy; ++sy; }
        const float gy = clip ? (float)max(0, abs(oy) - 1) * wy : 0.f;
        const float r2 = cut2f - gz * gz - gy * gy;
        if (r2 < 0.f) continue;
        int ox_lo = (oz == 0 && oy == 0) ? 0 : -S, ox_hi = S;
        if (clip) {
          const int m = 1 + (int)floorf(sqrtf(r2) / wx);
          ox_lo = max(ox_lo, -m);
          ox_hi = min(ox_hi, m);
        }
        const int rowcell = g.cell0 + (rz * ncy + ry) * ncx;
        int ox = ox_lo;
        while (ox <= ox_hi) {
          int rx = cx + ox, sx = 0;
          while (rx < 0) { rx += ncx; --sx; }
          while (rx >= ncx) { rx -= ncx; ++sx; }
          int len = 1;
          while (ox + len <= ox_hi && rx + len < ncx) ++len;
          const int beg = d.cell_start[rowcell + rx];
          const int end = d.cell_start[rowcell + rx + len];
          ox += len;
          float shx, shy, shz;
          img_vec32(g, sx, sy, sz, shx, shy, shz);
          // image 0 arises only at offset (0, 0, ox >= 0): the partners of
          // an atom there are the atoms after it
          const bool self_img = (sx == 0 && sy == 0 && sz == 0);
          const uint32_t img = (uint32_t)img_pack(sx, sy, sz);
          const uint32_t img_m = (uint32_t)img_pack(-sx, -sy, -sz);
          for (int b0 = beg; b0 < end; b0 += TB) {
            const int nb = min(TB, end - b0);
            const int nrow = na + nb;
            __syncthreads();
            for (int k = tid; k < nb; k += TILE_T) {
              T.bx[k] = d.xs[b0 + k];
              T.bf[k] = d.xf[b0 + k];
              T.bl[k] = d.xl[b0 + k];
            }
            for (int k = tid; k < nrow; k += TILE_T) T.cnt[0][k] = T.cnt[1][k] = 0;
            if (tid == 0) T.nq = 0;
            __syncthreads();
            const int np = na * nb;
            for (int p0 = 0; p0 < np; p0 += TQ) {
              const int pe = min(np, p0 + TQ);
              // FP32 prefilter of the tile's pairs into the queue
              for (int p = p0 + tid; p < pe; p += TILE_T) {
                const int a = p / nb, b = p - a * nb;
                if (self_img && b0 + b <= a0 + a) continue;
                const float4 xa = T.af[a], xb = T.bf[b];
                const float fx = xb.x + shx - xa.x;
                const float fy = xb.y + shy - xa.y;
                const float fz = xb.z + shz - xa.z;
                if (fx * fx + fy * fy + fz * fz <= cut2f) {
                  const int slot = atomicAdd(&T.nq, 1);
                  T.q[slot] = ((uint32_t)a << 16) | (uint32_t)b;
                }
              }
              __syncthreads();
              const int nq = T.nq;
              // membership and near/far of each direction; rows' ranks
              for (int k = tid; k < nq; k += TILE_T) {
                const int a = (int)(T.q[k] >> 16), b = (int)(T.q[k] & 0xffffu);
                float dx, dy, dz;
                disp32(g, T.bf[b], T.bl[b], T.af[a], T.al[a], sx, sy, sz, dx, dy, dz);
                const float d2f = dx * dx + dy * dy + dz * dz;
                bool in = false, near = false, in_m = false, near_m = false;
                if (d2f <= lc2 * (1.f - MARGIN32)) {
                  in = in_m = true;
                } else if (d2f <= lc2 * (1.f + MARGIN32)) {
                  in = exact_d2v(T.bx[b], sx, sy, sz, T.ax[a], g) <= C.list_cut2;
                  in_m = exact_d2v(T.ax[a], -sx, -sy, -sz, T.bx[b], g) <= C.list_cut2;
                }
                if (MIXED) {
                  near = near_m = d2f <= nc2 * (1.f + MARGIN32);
                } else if (in || in_m) {
                  if (d2f <= nc2 * (1.f - MARGIN32)) {
                    near = near_m = true;
                  } else if (d2f <= nc2 * (1.f + MARGIN32)) {
                    near = near_exact(exact_d2v(T.bx[b], sx, sy, sz, T.ax[a], g), C);
                    near_m = near_exact(exact_d2v(T.ax[a], -sx, -sy, -sz, T.bx[b], g), C);
                  }
                }
                double d2 = 0.0;
                if (!MIXED && (in || in_m)) {
                  if (use_h_fp(d, C, g, d2f)) {
                    // r^2 as an FP32 pair, its bits in the FP64 slot
                    const fpair p = fp_d2(g, T.bf[b], T.bl[b], T.af[a], T.al[a], sx, sy, sz);
                    d2 = __hiloint2double(__float_as_int(p.hi), __float_as_int(p.lo));
                  } else {
                    double ex, ey, ez;
                    disp64(g, T.bx[b], T.ax[a], sx, sy, sz, ex, ey, ez);
                    d2 = fma(ex, ex, fma(ey, ey, ez * ez));
                  }
                }
                T.d2[k] = d2;
                T.d2f[k] = d2f;
                T.fl[k] = (unsigned char)((in ? 1 : 0) | (near ? 2 : 0) | (in_m ? 4 : 0) |
                                          (near_m ? 8 : 0));
                T.rk[k][0] = in ? (unsigned short)atomicAdd(&T.cnt[near ? 0 : 1][a], 1) : 0;
                T.rk[k][1] = in_m ? (unsigned short)atomicAdd(&T.cnt[near_m ? 0 : 1][na + b], 1) : 0;
              }
              __syncthreads();
              // claim each row part's slots once per tile pass
              for (int k = tid; k < 2 * nrow; k += TILE_T) {
                const int part = k / nrow, t = k - part * nrow;
                const int cnt = T.cnt[part][t];
                const int row = t < na ? a0 + t : b0 + (t - na);
                T.cnt[part][t] = cnt ? atomicAdd(part == 0 ? &d.n_near[row] : &d.n_far[row], cnt) : 0;
              }
              __syncthreads();
              // H once per pair, both entries
              for (int k = tid; k < nq; k += TILE_T) {
                const int a = (int)(T.q[k] >> 16), b = (int)(T.q[k] & 0xffffu);
                const int f = T.fl[k];
                if (!(f & 5)) continue;
                const int ta = __float_as_int(T.af[a].w), tb = __float_as_int(T.bf[b].w);
                double h;
                float h32;
                float2 hp = make_float2(0.f, 0.f);
                if (!MIXED && use_h_fp(d, C, g, T.d2f[k])) {
                  const double v = T.d2[k];
                  const fpair w = pair_h_fp(
                      d, C, ta, tb, {__int_as_float(__double2hiint(v)), __int_as_float(__double2loint(v))});
                  hp = make_float2(w.hi, w.lo);
                } else {
                  pair_h<MIXED>(d, C, F, ta, tb, T.d2[k], T.d2f[k], h, h32);
                  if (!MIXED) hp = h_pair(h);
                }
                if (f & 1) {
                  const bool nr = f & 2;
                  const int pos = T.cnt[nr ? 0 : 1][a] + T.rk[k][0];
                  if (pos < (nr ? capN : capF)) {
                    const long long slot = (long long)(a0 + a) * d.nb_cap + (nr ? pos : capN + pos);
                    d.nbr[slot] = ((uint32_t)(b0 + b) << 8) | img;
                    if (MIXED) d.hval32[slot] = h32;
                    else d.hvalp[slot] = hp;
                  }
                }
                if (f & 4) {
                  const bool nr = f & 8;
                  const int pos = T.cnt[nr ? 0 : 1][na + b] + T.rk[k][1];
                  if (pos < (nr ? capN : capF)) {
                    const long long slot = (long long)(b0 + b) * d.nb_cap + (nr ? pos : capN + pos);
                    d.nbr[slot] = ((uint32_t)(a0 + a) << 8) | img_m;
                    if (MIXED) d.hval32[slot] = h32;
                    else d.hvalp[slot] = hp;
                  }
                }
              }
              __syncthreads();
              for (int k = tid; k < nrow; k += TILE_T) T.cnt[0][k] = T.cnt[1][k] = 0;
              if (tid == 0) T.nq = 0;
              __syncthreads();
            }
          }
        }
      }
    }
  }
}

// after the build: rows whose parts overflowed their capacity, and the
// largest part sizes (the host regrows to them and re-runs the build)
__global__ void k_nbr_check(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int nn = 0, nf = 0;
  if (i < d.n) {
    nn = d.n_near[i];
    nf = d.n_far[i];
  }
  for (int off = 16; off > 0; off >>= 1) {
    nn = max(nn, __shfl_down_sync(FULL, nn, off));
    nf = max(nf, __shfl_down_sync(FULL, nf, off));
  }
  if ((threadIdx.x & 31) == 0) {
    if (nn > d.nb_capN || nf > d.nb_cap - d.nb_capN) atomicOr(&d.status[ST_OVF], OVF_NBR);
    atomicMax(&d.status[ST_MAXNB], nn);
    atomicMax(&d.status[ST_MAXNF], nf);
  }
}

// -------------------------------------------------------------------
// bond list with uncorrected bond orders, and H-bond partners
//
// One warp per atom i over the near part of its row.  H-bond partners are
// decided from the FP32 (hi, lo) distance away from hbond_cut and from the
// exact distance near it.  Bond candidates (d <= bond_cut)
// whose FP32 estimate of BO' is above half of bo_cut (FP32 errors are ~1e-4
// relative here) are written to the bond slots of i; k_bond_prime then
// evaluates BO' and the exact BO' >= bo_cut decision one thread per
// candidate (a row has only a few candidates, so a per-row warp would run
// the FP64 pow/exp with most lanes idle), and k_bond_finish compacts the
// rows and sums dDeltap and the total bond order.

// BO' terms in FP64: (d / r)^p as exp(p (log d - log r)) with log d once
// per bond and log r from the control block (a few 1e-16 relative from pow,
// far inside the 1e-10 bond-order bars; the reference's live form is a
// polynomial pow/exp on the CPEs)
__device__ __forceinline__ void bo_prime64(const Control &C, int ti, int tj, const Sbp &si,
                                           const Sbp &sj, const Tbp &tw, double dist,
                                           double &BOs, double &BOpi, double &BOpi2,
                                           double &C12, double &C34, double &C56) {
  BOs = BOpi = BOpi2 = C12 = C34 = C56 = 0;
  const double ld = log(dist);
  const double *lr = C.ln_r[ti][tj];
  if (si.r_s > 0.0 && sj.r_s > 0.0) {
    C12 = tw.p_bo1 * exp(tw.p_bo2 * (ld - lr[0]));
    BOs = (1.0 + C.bo_cut) * exp(C12);
  }
  if (si.r_pi > 0.0 && sj.r_pi > 0.0) {
    C34 = tw.p_bo3 * exp(tw.p_bo4 * (ld - lr[1]));
    BOpi = exp(C34);
  }
  if (si.r_pi_pi > 0.0 && sj.r_pi_pi > 0.0) {
    C56 = tw.p_bo5 * exp(tw.p_bo6 * (ld - lr[2]));
    BOpi2 = exp(C56);
  }
}

// BO' of the bond candidates, 32 candidates of a warp's 32 atoms at a time
// (warp_items), so the FP64 log/exp run with full warps instead of the few
// lanes a per-atom warp has candidates for.  Accepted entries get their exact
// distance, bond orders and dBO' terms; rejected ones (d > bond_cut or
// BO' < bo_cut) are marked with a negative distance and removed by
// k_bond_finish.  Both forms take the exact FP64 distance and FP64 BO':
// BO' = exp(p_bo1 (d/r)^p_bo2) amplifies relative errors of d by
// |p_bo1 p_bo2 (d/r)^p_bo2| (up to ~10 for C-C and C-N bonds), and in FP32
// that left the mixed form's forces on the TATB crystal 1.7e-4 (relative
// RMS) from the FP64 forces, against 1e-5 with FP64 BO'.
// BO' is symmetric in the pair.  The candidate of a pair that sorts first
// (lower atom, then lower image code) evaluates it and fills both
// directions' slots; the other finds its partner's slot and leaves it.  A
// candidate whose mirror is not listed evaluates its own slot.
// Returns the mirror slot (or -1) and whether this candidate evaluates.
__device__ __forceinline__ long long bond_mirror(const Dev &d, int i, int k, bool &work) {
  const int n = d.n;
  const uint32_t e = d.b_nbr[(long long)k * n + i];
  const int j = (int)(e >> 8);
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const uint32_t want = ((uint32_t)i << 8) | (uint32_t)img_pack(-sx, -sy, -sz);
  const int nbj = min(d.nbonds[j], d.bond_cap);
  long long m = -1;
  for (int q = 0; q < nbj; ++q)
    if (d.b_nbr[(long long)q * n + j] == want) {
      m = (long long)q * n + j;
      break;
    }
  const bool owner = j > i || (j == i && (e & 255u) < (want & 255u));
  work = owner || m < 0;
  return m;
}

// one candidate's BO' (and its mirror slot m when m >= 0)
__device__ __forceinline__ void bond_prime_item(const Dev &d, int i, int k, long long m) {
  const int n = d.n;
  const Control &C = *d.ctl;
  const ForceField &F = *d.ff;
  const long long s = (long long)k * n + i;
  const long long S3 = (long long)d.bond_cap * n;
  const uint32_t e = d.b_nbr[s];
  const int j = (int)(e >> 8);
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const SegGeom &g = d.seg[d.seg_s[i]];
  double dx, dy, dz;
  disp64(g, d.xs[j], d.xs[i], sx, sy, sz, dx, dy, dz);
  const double dist =
      __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  if (!(dist <= C.bond_cut)) {
    d.b_d[s] = -1.0;
    if (m >= 0) d.b_d[m] = -1.0;
    return;
  }
  const int ti = d.ts[i], tj = d.ts[j];
  const Sbp &si = F.sbp[ti], &sj = F.sbp[tj];
  const Tbp &tw = F.tbp[ti][tj];
  double BOs, BOpi, BOpi2, C12, C34, C56;
  bo_prime64(C, ti, tj, si, sj, tw, dist, BOs, BOpi, BOpi2, C12, C34, C56);
  if (!((BOs + BOpi + BOpi2) >= C.bo_cut)) {
    d.b_d[s] = -1.0;
    if (m >= 0) d.b_d[m] = -1.0;
    return;
  }
  const double r2 = dist * dist;
  const double Cs = tw.p_bo2 * C12 / r2;
  const double Cpi = tw.p_bo4 * C34 / r2;
  const double Cpi2 = tw.p_bo6 * C56 / r2;
  const double gb = -(BOs * Cs + BOpi * Cpi + BOpi2 * Cpi2);
  const double api = -BOpi * Cpi, api2 = -BOpi2 * Cpi2;
  // this direction with (dx, dy, dz), the mirror with it negated
  for (int side = 0; side < (m >= 0 ? 2 : 1); ++side) {
    const long long t = side ? m : s;
    const double sg = side ? -1.0 : 1.0;
    const double ex = sg * dx, ey = sg * dy, ez = sg * dz;
    d.b_d[t] = dist;
    d.b_dx[t] = ex; d.b_dy[t] = ey; d.b_dz[t] = ez;
    d.b_BO[t] = BOs + BOpi + BOpi2 - C.bo_cut;
    d.b_BOs[t] = BOs - C.bo_cut;
    d.b_BOpi[t] = BOpi;
    d.b_BOpi2[t] = BOpi2;
    d.b_dBOp[t] = gb * ex; d.b_dBOp[S3 + t] = gb * ey; d.b_dBOp[2 * S3 + t] = gb * ez;
    d.b_dlnpi[t] = api * ex; d.b_dlnpi[S3 + t] = api * ey; d.b_dlnpi[2 * S3 + t] = api * ez;
    d.b_dlnpi2[t] = api2 * ex; d.b_dlnpi2[S3 + t] = api2 * ey; d.b_dlnpi2[2 * S3 + t] = api2 * ez;
    d.b_Cdbo[t] = 0.0; d.b_Cdbopi[t] = 0.0; d.b_Cdbopi2[t] = 0.0;
  }
}

struct BondQueue {
  int i[64], k[64];
  long long m[64];
};

// One warp per 32 atoms over all their candidates (warp_items): the
// candidates that evaluate go to a per-warp queue and are evaluated 32 at
// a time, so the FP64 log/exp run with full warps
__global__ void __launch_bounds__(256) k_bond_prime(Dev d) {
  __shared__ BondQueue queues[8];
  BondQueue &Q = queues[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = i < d.n ? min(d.nbonds[i], d.bond_cap) : 0;
  int qn = 0;
  auto drain = [&](bool all) {
    while (qn >= 32 || (all && qn > 0)) {
      const int c = min(qn, 32);
      if (lane < c) bond_prime_item(d, Q.i[lane], Q.k[lane], Q.m[lane]);
      __syncwarp();
      const int left = qn - c;
      int li = 0, lk = 0;
      long long lm = 0;
      if (lane < left) {
        li = Q.i[c + lane];
        lk = Q.k[c + lane];
        lm = Q.m[c + lane];
      }
      __syncwarp();
      if (lane < left) {
        Q.i[lane] = li;
        Q.k[lane] = lk;
        Q.m[lane] = lm;
      }
      __syncwarp();
      qn = left;
    }
  };
  warp_items_all(cnt, i, [&](bool has, int a, int k) {
    bool work = false;
    long long m = -1;
    if (has) m = bond_mirror(d, a, k, work);
    const unsigned mw = __ballot_sync(0xffffffffu, work);
    if (work) {
      const int slot = qn + __popc(mw & ((1u << lane) - 1u));
      Q.i[slot] = a;
      Q.k[slot] = k;
      Q.m[slot] = m;
    }
    qn += __popc(mw);
    __syncwarp();
    drain(false);
  });
  drain(true);
}

// per atom: drop rejected candidates (keeping the order of the rest), then
// the bond count, sum_j dBO'_ij (dDeltap) and the total bond order, summed
// in slot order
__global__ void k_bond_finish(Dev d) {
  const int n = d.n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nc = min(d.nbonds[i], d.bond_cap);
  const long long S3 = (long long)d.bond_cap * n;
  double ddx = 0.0, ddy = 0.0, ddz = 0.0, bsum = 0.0;
  int w = 0;
  for (int k = 0; k < nc; ++k) {
    const long long s = (long long)k * n + i;
    if (d.b_d[s] < 0.0) continue;
    if (w != k) {
      const long long t = (long long)w * n + i;
      d.b_nbr[t] = d.b_nbr[s];
      d.b_d[t] = d.b_d[s];
      d.b_dx[t] = d.b_dx[s]; d.b_dy[t] = d.b_dy[s]; d.b_dz[t] = d.b_dz[s];
      d.b_BO[t] = d.b_BO[s]; d.b_BOs[t] = d.b_BOs[s];
      d.b_BOpi[t] = d.b_BOpi[s]; d.b_BOpi2[t] = d.b_BOpi2[s];
      for (int c = 0; c < 3; ++c) {
        d.b_dBOp[c * S3 + t] = d.b_dBOp[c * S3 + s];
        d.b_dlnpi[c * S3 + t] = d.b_dlnpi[c * S3 + s];
        d.b_dlnpi2[c * S3 + t] = d.b_dlnpi2[c * S3 + s];
      }
      d.b_Cdbo[t] = 0.0; d.b_Cdbopi[t] = 0.0; d.b_Cdbopi2[t] = 0.0;
    }
    const long long t = (long long)w * n + i;
    ddx += d.b_dBOp[t];
    ddy += d.b_dBOp[S3 + t];
    ddz += d.b_dBOp[2 * S3 + t];
    bsum += d.b_BO[t];
    ++w;
  }
  // an overflowed row (more candidates than slots) keeps its candidate
  // count, so the host sees the overflow and rebuilds with more slots
  if (d.nbonds[i] <= d.bond_cap) d.nbonds[i] = w;
  d.dDeltap[i] = ddx;
  d.dDeltap[n + i] = ddy;
  d.dDeltap[2 * n + i] = ddz;
  d.bo0[i] = bsum;
}

template <bool MIXED>
__global__ void __launch_bounds__(NB_WARPS * 32) k_build_bonds(Dev d) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= d.n) return;
  const Control &C = *d.ctl;
  const ForceField &F = *d.ff;
  const double4 xi = d.xs[i];
  const float4 xif = d.xf[i];
  const int ti = d.ts[i];
  const Sbp &si = F.sbp[ti];
  const bool ihb = (si.p_hbond == 1) && C.hbond_cut > 0.0;
  const long long row = (long long)i * d.nb_cap;
  const int nn = nbr_near_count(d, i);
  const int n = d.n;
  const SegGeom &g = d.seg[d.seg_s[i]];
  const float4 xil = d.xl[i];
  // FP32 prefilter radii: anything that could be within bond_cut, and for
  // an H atom's acceptor partners within hbond_cut
  const float rpb = (float)(C.bond_cut + 0.01), rph = (float)(fmax(C.bond_cut, C.hbond_cut) + 0.01);
  const float rpre2b = rpb * rpb, rpre2h = rph * rph;
  const float bo_half = C.bo_half_f;
  int nb = 0, nh = 0;
  // the next batch's entry and partner position are loaded while this
  // batch is tested
  uint32_t e_nx = 0;
  float4 xjf_nx = make_float4(0.f, 0.f, 0.f, 0.f);
  if (lane < nn) {
    e_nx = d.nbr[row + lane];
    xjf_nx = d.xf[e_nx >> 8];
  }
  for (int base = 0; base < nn; base += 32) {
    {
      const int p = base + lane;
      bool ish = false, cand = false;
      const uint32_t e = e_nx;
      const float4 xjf = xjf_nx;
      if (p + 32 < nn) {
        e_nx = d.nbr[row + p + 32];
        xjf_nx = d.xf[e_nx >> 8];
      }
      if (p < nn) {
        const int j = (int)(e >> 8);
        int sx, sy, sz;
        img_unpack((int)(e & 255u), &sx, &sy, &sz);
        float vx, vy, vz;
        img_vec32(g, sx, sy, sz, vx, vy, vz);
        const float fx = xjf.x + vx - xif.x;
        const float fy = xjf.y + vy - xif.y;
        const float fz = xjf.z + vz - xif.z;
        const int tj = __float_as_int(xjf.w);
        const bool hb_rel = ihb && F.sbp[tj].p_hbond == 2;
        if (fx * fx + fy * fy + fz * fz <= (hb_rel ? rpre2h : rpre2b)) {
          // FP32 distance from the (hi, lo) positions (a few FP32 ulps of
          // the displacement) decides away from the cutoffs; the exact
          // distance only within MARGIN32 of the H-bond cutoff.  Possible
          // bonds are decided exactly (and their values computed) by
          // k_bond_prime.
          const float4 lj = d.xl[j];
          float ex, ey, ez;
          disp32(g, xjf, lj, xif, xil, sx, sy, sz, ex, ey, ez);
          const float df = sqrtf(ex * ex + ey * ey + ez * ez);
          const float bc = C.bond_cut_f, hc = C.hbond_cut_f;
          if (hb_rel && fabsf(df - hc) <= MARGIN32 * hc) {
            double ax, ay, az;
            disp64(g, d.xs[j], xi, sx, sy, sz, ax, ay, az);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az));
            ish = __dsqrt_rn(d2) <= C.hbond_cut;
          } else {
            ish = hb_rel && df <= hc;
          }
          if (df <= bc * (1.f + MARGIN32)) {
            // with the hardware exp2/log2 (relative errors ~1e-6, against
            // the factor 2 between bo_half and bo_cut)
            const Control::BoEst &be = C.bo_est[ti][tj];
            const float lg = __log2f(df);
            float est = 0.f;
            if (be.mask & 1) est += C.bo_scale_f * exp2f(be.e[0] * exp2f(be.q[0] * (lg - be.l[0])));
            if (be.mask & 2) est += exp2f(be.e[1] * exp2f(be.q[1] * (lg - be.l[1])));
            if (be.mask & 4) est += exp2f(be.e[2] * exp2f(be.q[2] * (lg - be.l[2])));
            cand = est >= bo_half;
          }
        }
      }
      const unsigned mh = __ballot_sync(FULL, ish);
      if (ish) {
        const int k = nh + __popc(mh & lanemask_lt());
        if (k < d.hb_cap) d.hb_nbr[(long long)i * d.hb_cap + k] = e;
      }
      nh += __popc(mh);
      // candidates go to the bond slots in row order; k_bond_prime gives
      // them their FP64 BO' and k_bond_finish drops the rejected
      const unsigned mc = __ballot_sync(FULL, cand);
      if (cand) {
        const int k = nb + __popc(mc & lanemask_lt());
        if (k < d.bond_cap) d.b_nbr[(long long)k * n + i] = e;
      }
      nb += __popc(mc);
    }
  }
  if (lane == 0) {
    d.nbonds[i] = nb;
    d.nhb[i] = nh;
    if (nb > d.bond_cap) atomicOr(&d.status[ST_OVF], OVF_BOND);
    if (nh > d.hb_cap) atomicOr(&d.status[ST_OVF], OVF_HB);
    atomicMax(&d.status[ST_MAXB], nb);
    atomicMax(&d.status[ST_MAXHB], nh);
  }
}

// symmetric partner of each bond: (j -> i, -image) in j's list
__global__ void k_bond_sym(Dev d) {
  const int n = d.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t % n), k = (int)(t / n);
  if (k >= d.bond_cap || i >= n) return;
  if (k >= d.nbonds[i]) return;
  const long long s = (long long)k * n + i;
  const uint32_t e = d.b_nbr[s];
  const int j = (int)(e >> 8);
  int sx, sy, sz;
  img_unpack((int)(e & 255u), &sx, &sy, &sz);
  const uint32_t want = ((uint32_t)i << 8) | (uint32_t)img_pack(-sx, -sy, -sz);
  const int nbj = min(d.nbonds[j], d.bond_cap);
  int sym = -1;
  for (int q = 0; q < nbj; ++q)
    if (d.b_nbr[(long long)q * n + j] == want) sym = q * n + j;
  d.b_sym[s] = sym;
}

// list sizes for the statistics (status slots 5..7)
__global__ void k_count(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int a = 0, b = 0, c = 0;
  if (i < d.n) {
    a = d.n_near[i] + d.n_far[i];
    b = d.nbonds[i];
    c = d.nhb[i];
  }
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(FULL, a, off);
    b += __shfl_down_sync(FULL, b, off);
    c += __shfl_down_sync(FULL, c, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&d.status[5], a);
    atomicAdd(&d.status[6], b);
    atomicAdd(&d.status[7], c);
  }
}

}  // namespace

// exclusive scan of n ints (n < 2^30); bsum needs (n + 1023) / 1024 ints
void launch_scan(const int *in, int *out, int n, int *bsum, cudaStream_t st) {
  const int nb = (n + 1023) / 1024;
  k_scan_blocks<<<nb, 1024, 0, st>>>(in, out, bsum, n);
  k_scan_sums<<<1, 1024, 0, st>>>(bsum, nb, nullptr);
  k_scan_add<<<nb, 1024, 0, st>>>(out, bsum, n);
}

void launch_count(const Dev &d, cudaStream_t st) {
  k_count<<<(d.n + 255) / 256, 256, 0, st>>>(d);
}

void launch_bin_sort(const Dev &d, cudaStream_t st) {
  const int ncell = d.ncell;
  cudaMemsetAsync(d.cell_count, 0, sizeof(int) * (ncell + 1), st);
  cudaMemsetAsync(d.cell_fill, 0, sizeof(int) * (ncell + 1), st);
  const int B = 256;
  k_cell_assign<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  const int nb = (ncell + 1 + 1023) / 1024;
  // block sums live after the cell_fill counters
  int *bsum = d.cell_fill + (ncell + 1);
  k_scan_blocks<<<nb, 1024, 0, st>>>(d.cell_count, d.cell_start, bsum, ncell + 1);
  k_scan_sums<<<1, 1024, 0, st>>>(bsum, nb, nullptr);
  k_scan_add<<<nb, 1024, 0, st>>>(d.cell_start, bsum, ncell + 1);
  k_scatter<<<(d.n + B - 1) / B, B, 0, st>>>(d);
  k_cell_order<<<(ncell + B - 1) / B, B, 0, st>>>(d, ncell);
  k_gather<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

void launch_build_nbrs(const Dev &d, cudaStream_t st) {
  const int B = NB_WARPS * 32;
  const long long threads = (long long)d.n * 32;
  const unsigned G = (unsigned)((threads + B - 1) / B);
  // the part counters are claimed atomically by the build
  cudaMemsetAsync(d.n_near, 0, sizeof(int) * (size_t)d.n, st);
  cudaMemsetAsync(d.n_far, 0, sizeof(int) * (size_t)d.n, st);
  if (d.nbr_tiles) {
    if (d.mixed) k_build_nbrs_tiles<true><<<d.ncell, TILE_T, 0, st>>>(d);
    else k_build_nbrs_tiles<false><<<d.ncell, TILE_T, 0, st>>>(d);
  } else {
    if (d.mixed) k_build_nbrs<true><<<G, B, 0, st>>>(d);
    else k_build_nbrs<false><<<G, B, 0, st>>>(d);
  }
  k_nbr_check<<<(d.n + 255) / 256, 256, 0, st>>>(d);
}

void launch_build_bonds(const Dev &d, cudaStream_t st) {
  const long long threads = (long long)d.n * 32;
  const unsigned G = (unsigned)((threads + NB_WARPS * 32 - 1) / (NB_WARPS * 32));
  if (d.mixed) k_build_bonds<true><<<G, NB_WARPS * 32, 0, st>>>(d);
  else k_build_bonds<false><<<G, NB_WARPS * 32, 0, st>>>(d);
  k_bond_prime<<<(unsigned)((d.n + 255) / 256), 256, 0, st>>>(d);
  k_bond_finish<<<(d.n + 255) / 256, 256, 0, st>>>(d);
  const long long slots = (long long)d.n * d.bond_cap;
  k_bond_sym<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(d);
}

void launch_zero(void *p, size_t bytes, cudaStream_t st) { cudaMemsetAsync(p, 0, bytes, st); }
