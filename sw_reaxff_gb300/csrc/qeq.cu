// QEq charge equilibration: the s and t systems of the reference solved
// together ("dual"), each with a Jacobi-preconditioned CG that keeps the
// set-up, stopping test and iteration count of the reference's CG_v2.
//
//  k_qeq_setup   init_matvec: Jacobi diagonal, b_s = -chi, b_t = -1, cubic
//                (s) / quadratic (t) extrapolation from the 5-deep
//                histories (fix_qeq_reax_sunway.cpp:618-723)
//  k_spmvp, k_spmv32  sparse_matvec: b_i = eta_i x_i + sum_j H_ij x_j over
//                the full rows (fix_qeq_reax_sw64.c:357-498), both systems
//                per read of H, in compensated FP32 arithmetic (FP64 form:
//                H as an FP32 pair; mixed form: H in FP32)
//  k_cg_*, k_pcg_*  CG_v2 (fix_qeq_reax_sunway.cpp:983-1167): Jacobi PCG
//                with CG_v2's set-up, stopping test and iteration count, in
//                the standard (not pipelined) recurrences; a system that
//                has converged stops updating, so each keeps the iterate
//                and iteration count of a solve on its own
//  k_qeq_finish  calculate_Q (fix_qeq_reax_sunway.cpp:1697-1755)
#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;

// scalar slots in d.red (pairs: [s, t])
enum {
  R_ACC0 = 0, R_ACC1 = 2, R_BETA = 10, R_RHO = 12, R_BNORM = 16, R_ACTIVE = 20, R_ITERS = 22,
  R_SUM = 24, R_TOL = 26, R_IMAX = 27, R_INIT = 68
};
// (per segment: d.red + seg * RG_NRED; ACC0: p.q, ACC1: u.r of the
// iteration; R_INIT..R_INIT+3: the set-up sums b.b, u.r)

__device__ __forceinline__ int seg_at(const Dev &d, int s) { return s < d.n ? d.seg_s[s] : -1; }

// zero count slots from slot of every segment
__global__ void k_seg_zero(Dev d, int slot, int count) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nseg) return;
  for (int c = 0; c < count; ++c) d.red[(long long)g * RG_NRED + slot + c] = 0.0;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  return v;
}

__global__ void k_qeq_setup(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const int n = d.n, i = d.perm[s];
  const Sbp &sb = d.ff->sbp[d.ts[s]];
  d.Hdia_inv[s] = 1. / sb.eta;
  d.qb[s] = make_double2(-sb.chi, -1.0);
  const double *sh = d.s_hist, *th = d.t_hist;
  const double s0 = 4 * (sh[0 * n + i] + sh[2 * n + i]) - (6 * sh[1 * n + i] + sh[3 * n + i]);
  const double t0 = th[2 * n + i] + 3 * (th[0 * n + i] - th[1 * n + i]);
  d.qx[s] = make_double2(s0, t0);
}

// y = H x (+ eta x on the diagonal), one warp per row; FP64 form.  In the
// CG iterations (use_act) a system whose solve has converged is skipped:
// its half of y is not read again
// mixed form: the FP32 H with compensated FP32 arithmetic.  The vector is
// read as FP32 (hi, lo) pairs (x = hi + lo to ~2^-48), each product is
// formed exactly as p + e (fmaf) plus h*lo, and the row sum is carried as an
// unevaluated FP32 pair with Knuth's TwoSum, across the warp too; the pair
// becomes FP64 once per row.  The sums so carry ~46 significant bits: the
// CG then follows the FP64 iterates (it stagnates with plain FP32 sums),
// while reading 8 bytes of H and index per entry and running on the FP32
// units.
// (explicitly rounded operations: no contraction into FMAs may change them)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) += h * (xh + xl)
__device__ __forceinline__ void df_fma(float h, float xh, float xl, float &sh, float &sl) {
  const float p = __fmul_rn(h, xh);
  float e = __fmaf_rn(h, xh, -p);   // exact: h*xh = p + e
  e = __fmaf_rn(h, xl, e);
  float s, err;
  two_sum(sh, p, s, err);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

__device__ __forceinline__ void df_add(float &sh, float &sl, float oh, float ol) {
  float s, err;
  two_sum(sh, oh, s, err);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(err, ol));
}

__device__ __forceinline__ float4 split4(double2 v) {
  const float sh = __double2float_rn(v.x), th = __double2float_rn(v.y);
  return make_float4(sh, __double2float_rn(v.x - (double)sh), th, __double2float_rn(v.y - (double)th));
}

// RW lanes per row (rows average several hundred entries), each keeping
// the s and t sums of its entries.  The compensated pairs of the two
// systems are reduced together (the first exchange swaps halves, each later
// level is one compensated add per lane), and lanes 0 and 1 of the row
// group finish y_s and y_t: the FP64 tail (conversion, eta x) is one warp
// instruction sequence for four values, not eight per row.
template <int RW>
__device__ __forceinline__ void df_pair_sum(float &vh, float &vl, float ah, float al, float bh,
                                            float bl, int gl) {
  const bool odd = gl & 1;
  vh = odd ? bh : ah;
  vl = odd ? bl : al;
  const float oh = __shfl_xor_sync(FULL, odd ? ah : bh, 1);
  const float ol = __shfl_xor_sync(FULL, odd ? al : bl, 1);
  df_add(vh, vl, oh, ol);
  for (int off = 2; off < RW; off <<= 1) {
    const float ph = __shfl_xor_sync(FULL, vh, off), pl = __shfl_xor_sync(FULL, vl, off);
    df_add(vh, vl, ph, pl);
  }
}

template <int RW>
__global__ void __launch_bounds__(256) k_spmv32(Dev d, const double2 *__restrict__ x, double2 *__restrict__ y,
                                                int use_act) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int gl = (int)(tid & (RW - 1));
  const int i = (int)(tid / RW);
  const bool valid = i < d.n;     // no early return: the row group shuffles
  const long long row = (long long)i * d.nb_cap;
  const int nn = valid ? nbr_near_count(d, i) : 0, nf = valid ? nbr_far_count(d, i) : 0;
  const int tot = nn + nf, capN = d.nb_capN;
  const float4 *__restrict__ x32 = d.qd32;
  bool on_s = valid, on_t = valid;
  if (use_act && valid) {
    // activity flags are exactly 0.0 or 1.0: compare their bits (no FP64)
    const long long *R = reinterpret_cast<const long long *>(d.red + (long long)d.seg_s[i] * RG_NRED);
    on_s = R[R_ACTIVE] != 0;
    on_t = R[R_ACTIVE + 1] != 0;
  }
  float sh = 0.f, sl = 0.f, th = 0.f, tl = 0.f;
  if (on_s && on_t) {
    // four entries per lane and step: their index and H loads, then their
    // four gathers of x, are in flight together; two compensated sums per
    // system
    float sh1 = 0.f, sl1 = 0.f, th1 = 0.f, tl1 = 0.f;
    int p = gl;
    for (; p + 3 * RW < tot; p += 4 * RW) {
      uint32_t e4[4];
      float h4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = p + u * RW;
        const int s = q < nn ? q : capN + (q - nn);
        e4[u] = d.nbr[row + s];
        h4[u] = d.hval32[row + s];
      }
      float4 x4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x4[u] = x32[e4[u] >> 8];
      df_fma(h4[0], x4[0].x, x4[0].y, sh, sl);
      df_fma(h4[0], x4[0].z, x4[0].w, th, tl);
      df_fma(h4[1], x4[1].x, x4[1].y, sh1, sl1);
      df_fma(h4[1], x4[1].z, x4[1].w, th1, tl1);
      df_fma(h4[2], x4[2].x, x4[2].y, sh, sl);
      df_fma(h4[2], x4[2].z, x4[2].w, th, tl);
      df_fma(h4[3], x4[3].x, x4[3].y, sh1, sl1);
      df_fma(h4[3], x4[3].z, x4[3].w, th1, tl1);
    }
    for (; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const uint32_t e = d.nbr[row + slot];
      const float h = d.hval32[row + slot];
      const float4 xj = x32[e >> 8];
      df_fma(h, xj.x, xj.y, sh, sl);
      df_fma(h, xj.z, xj.w, th, tl);
    }
    df_add(sh, sl, sh1, sl1);
    df_add(th, tl, th1, tl1);
  } else if (on_s) {
    for (int p = gl; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const float h = d.hval32[row + slot];
      const float4 xj = x32[d.nbr[row + slot] >> 8];
      df_fma(h, xj.x, xj.y, sh, sl);
    }
  } else if (on_t) {
    for (int p = gl; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const float h = d.hval32[row + slot];
      const float4 xj = x32[d.nbr[row + slot] >> 8];
      df_fma(h, xj.z, xj.w, th, tl);
    }
  }
  float vh, vl;
  df_pair_sum<RW>(vh, vl, sh, sl, th, tl, gl);
  if (valid && gl < 2) {
    const double eta = d.ff->sbp[d.ts[i]].eta;
    const double *xi = reinterpret_cast<const double *>(x) + 2 * (long long)i;
    reinterpret_cast<double *>(y)[2 * (long long)i + gl] = fma(eta, xi[gl], (double)vh + (double)vl);
  }
}


// (sh, sl) += (hh + hl) * (xh + xl): the leading product exact (fmaf), the
// cross terms hh xl and hl xh added to its error (hl xl, ~2^-48 of the
// product, is left out)
__device__ __forceinline__ void dd_fma(float hh, float hl, float xh, float xl, float &sh, float &sl) {
  const float p = __fmul_rn(hh, xh);
  float e = __fmaf_rn(hh, xh, -p);
  e = __fmaf_rn(hh, xl, e);
  e = __fmaf_rn(hl, xh, e);
  float s, err;
  two_sum(sh, p, s, err);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// FP64 form: H_ij stored as an FP32 pair (its table value to ~2^-48) times
// the vector's FP32 (hi, lo) pairs, summed as in k_spmv32: the products and
// sums keep ~2^-46 of |H||x| (the FP64 DFMA form's 2^-53 is not needed by a
// solve to 1e-6, and GB300 runs FP64 FMAs at 1/64 of the FP32 rate).
// 12 bytes of index and H per entry.
template <int RW>
__global__ void __launch_bounds__(256) k_spmvp(Dev d, const double2 *__restrict__ x, double2 *__restrict__ y,
                                               int use_act) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int gl = (int)(tid & (RW - 1));
  const int i = (int)(tid / RW);
  const bool valid = i < d.n;     // no early return: the row group shuffles
  const long long row = (long long)i * d.nb_cap;
  const int nn = valid ? nbr_near_count(d, i) : 0, nf = valid ? nbr_far_count(d, i) : 0;
  const int tot = nn + nf, capN = d.nb_capN;
  const float4 *__restrict__ x32 = d.qd32;
  const float2 *__restrict__ H = d.hvalp;
  bool on_s = valid, on_t = valid;
  if (use_act && valid) {
    const long long *R = reinterpret_cast<const long long *>(d.red + (long long)d.seg_s[i] * RG_NRED);
    on_s = R[R_ACTIVE] != 0;
    on_t = R[R_ACTIVE + 1] != 0;
  }
  float sh = 0.f, sl = 0.f, th = 0.f, tl = 0.f;
  if (on_s && on_t) {
    float sh1 = 0.f, sl1 = 0.f, th1 = 0.f, tl1 = 0.f;
    int p = gl;
    for (; p + 3 * RW < tot; p += 4 * RW) {
      uint32_t e4[4];
      float2 h4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = p + u * RW;
        const int s = q < nn ? q : capN + (q - nn);
        e4[u] = d.nbr[row + s];
        h4[u] = H[row + s];
      }
      float4 x4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x4[u] = x32[e4[u] >> 8];
      dd_fma(h4[0].x, h4[0].y, x4[0].x, x4[0].y, sh, sl);
      dd_fma(h4[0].x, h4[0].y, x4[0].z, x4[0].w, th, tl);
      dd_fma(h4[1].x, h4[1].y, x4[1].x, x4[1].y, sh1, sl1);
      dd_fma(h4[1].x, h4[1].y, x4[1].z, x4[1].w, th1, tl1);
      dd_fma(h4[2].x, h4[2].y, x4[2].x, x4[2].y, sh, sl);
      dd_fma(h4[2].x, h4[2].y, x4[2].z, x4[2].w, th, tl);
      dd_fma(h4[3].x, h4[3].y, x4[3].x, x4[3].y, sh1, sl1);
      dd_fma(h4[3].x, h4[3].y, x4[3].z, x4[3].w, th1, tl1);
    }
    for (; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const uint32_t e = d.nbr[row + slot];
      const float2 h = H[row + slot];
      const float4 xj = x32[e >> 8];
      dd_fma(h.x, h.y, xj.x, xj.y, sh, sl);
      dd_fma(h.x, h.y, xj.z, xj.w, th, tl);
    }
    df_add(sh, sl, sh1, sl1);
    df_add(th, tl, th1, tl1);
  } else if (on_s) {
    for (int p = gl; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const float2 h = H[row + slot];
      const float4 xj = x32[d.nbr[row + slot] >> 8];
      dd_fma(h.x, h.y, xj.x, xj.y, sh, sl);
    }
  } else if (on_t) {
    for (int p = gl; p < tot; p += RW) {
      const int slot = p < nn ? p : capN + (p - nn);
      const float2 h = H[row + slot];
      const float4 xj = x32[d.nbr[row + slot] >> 8];
      dd_fma(h.x, h.y, xj.z, xj.w, th, tl);
    }
  }
  float vh, vl;
  df_pair_sum<RW>(vh, vl, sh, sl, th, tl, gl);
  if (valid && gl < 2) {
    const double eta = d.ff->sbp[d.ts[i]].eta;
    const double *xi = reinterpret_cast<const double *>(x) + 2 * (long long)i;
    reinterpret_cast<double *>(y)[2 * (long long)i + gl] = fma(eta, xi[gl], (double)vh + (double)vl);
  }
}

// r = b - q; u = r*Hdia_inv; d = u
__global__ void k_cg_init1(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const double hi = d.Hdia_inv[s];
  const double2 b = d.qb[s], q = d.qq[s];
  const double2 r = make_double2(b.x - 1 * q.x, b.y - 1 * q.y);
  d.qr[s] = r;
  const double2 u = make_double2(r.x * hi, r.y * hi);
  d.qu[s] = u;
  d.qd[s] = u;
  if (d.qd32) d.qd32[s] = split4(u);
}

// set-up sums b.b and u.r (u = r Hdia_inv)
__global__ void k_cg_init_sums(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (s < d.n) {
    const double2 u = d.qu[s], r = d.qr[s], b = d.qb[s];
    v[0] = b.x * b.x; v[1] = b.y * b.y;
    v[2] = u.x * r.x; v[3] = u.y * r.y;
  }
  seg_block_add<4>(v, seg_at(d, s), d.red + R_INIT, RG_NRED);
}

// one thread per segment: |b|, rho = u.r, the first iteration's activity
// (iteration 1 is the set-up, as CG_v2 counts); counts the segments with
// an active solve
__global__ void k_cg_init_ctrl(Dev d, double tol, int imax) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nseg) return;
  double *R = d.red + (long long)g * RG_NRED;
  R[R_TOL] = tol;
  R[R_IMAX] = imax;
  for (int c = 0; c < 2; ++c) {
    const double bb = R[R_INIT + c], ur = R[R_INIT + 2 + c];
    R[R_BNORM + c] = sqrt(bb);
    R[R_RHO + c] = ur;
    R[R_BETA + c] = 0.0;
    R[R_ITERS + c] = 1.0;
    R[R_ACTIVE + c] = (1 < imax && sqrt(ur) / R[R_BNORM + c] > tol) ? 1.0 : 0.0;
    R[R_ACC0 + c] = 0.0;
    R[R_ACC1 + c] = 0.0;
  }
  if (R[R_ACTIVE] != 0.0 || R[R_ACTIVE + 1] != 0.0) atomicAdd(d.n_active, 1);
}

// Jacobi-preconditioned CG, per system and segment:
//   q = H p;  alpha = rho / p.q;  x += alpha p;  r -= alpha q;
//   u = r Hdia_inv;  rho' = u.r;  beta = rho' / rho;  p = u + beta p
// The reference's CG_v2 runs the pipelined form of these recurrences
// (Ghysels-Vanroose: two more products at the set-up, one reduction phase
// per iteration, to hide MPI reductions); in exact arithmetic both give the
// same iterates, residuals and iteration counts, and on one GPU the extra
// reduction phase costs a kernel boundary, not an SpMV.

// p = u + beta p (beta = 0 at the set-up, where p = u already); p is the
// SpMV's input (qd, and its split copy in the mixed form)
__global__ void k_pcg_p(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const double *R = d.red + (long long)d.seg_s[s] * RG_NRED;
  const bool as = R[R_ACTIVE] != 0.0, at = R[R_ACTIVE + 1] != 0.0;
  if (!(as || at)) return;
  const double2 u = d.qu[s];
  double2 p = d.qd[s];
  if (as) p.x = u.x + R[R_BETA] * p.x;
  if (at) p.y = u.y + R[R_BETA + 1] * p.y;
  d.qd[s] = p;
  if (d.qd32) d.qd32[s] = split4(p);
}

// p.q per segment (ACC0).  ONE: a single segment, taken by a grid-stride
// loop over ~600 blocks so the FP64 atomics come from few blocks.
template <bool ONE>
__global__ void k_pcg_sigma(Dev d) {
  double v[2] = {0, 0};
  int sg = -1;
  if (ONE) {
    const bool as = d.red[R_ACTIVE] != 0.0, at = d.red[R_ACTIVE + 1] != 0.0;
    if (as || at) {
      for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < d.n; s += gridDim.x * blockDim.x) {
        const double2 p = d.qd[s], q = d.qq[s];
        if (as) v[0] += p.x * q.x;
        if (at) v[1] += p.y * q.y;
      }
    }
    sg = 0;
  } else {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    sg = seg_at(d, s);
    if (sg >= 0) {
      const double *R = d.red + (long long)sg * RG_NRED;
      const double2 p = d.qd[s], q = d.qq[s];
      if (R[R_ACTIVE] != 0.0) v[0] = p.x * q.x;
      if (R[R_ACTIVE + 1] != 0.0) v[1] = p.y * q.y;
    }
  }
  seg_block_add<2>(v, sg, d.red + R_ACC0, RG_NRED);
}

// alpha = rho / p.q; x += alpha p; r -= alpha q; u = r Hdia_inv; u.r per
// segment (ACC1).  Clears the active count that k_pcg_ctrl recounts.
__device__ __forceinline__ void pcg_update(const Dev &d, int s, const double *R, bool as, bool at,
                                           double *v) {
  const double hi = d.Hdia_inv[s];
  const double2 p = d.qd[s], q = d.qq[s];
  double2 x = d.qx[s], r = d.qr[s], u = d.qu[s];
  if (as) {
    const double a = R[R_RHO] / R[R_ACC0];
    x.x += a * p.x; r.x -= a * q.x; u.x = r.x * hi;
    v[0] += u.x * r.x;
  }
  if (at) {
    const double a = R[R_RHO + 1] / R[R_ACC0 + 1];
    x.y += a * p.y; r.y -= a * q.y; u.y = r.y * hi;
    v[1] += u.y * r.y;
  }
  d.qx[s] = x; d.qr[s] = r; d.qu[s] = u;
}

template <bool ONE>
__global__ void k_pcg_update(Dev d) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *d.n_active = 0;
  double v[2] = {0, 0};
  int sg = -1;
  if (ONE) {
    const bool as = d.red[R_ACTIVE] != 0.0, at = d.red[R_ACTIVE + 1] != 0.0;
    if (as || at)
      for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < d.n; s += gridDim.x * blockDim.x)
        pcg_update(d, s, d.red, as, at, v);
    sg = 0;
  } else {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    sg = seg_at(d, s);
    if (sg >= 0) {
      const double *R = d.red + (long long)sg * RG_NRED;
      const bool as = R[R_ACTIVE] != 0.0, at = R[R_ACTIVE + 1] != 0.0;
      if (as || at) pcg_update(d, s, R, as, at, v);
    }
  }
  seg_block_add<2>(v, sg, d.red + R_ACC1, RG_NRED);
}

// one thread per segment: beta, the loop increment and the test of the
// next iteration (CG_v2's criterion sqrt(u.r) / |b| > tol), the active
// count
__global__ void k_pcg_ctrl(Dev d) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nseg) return;
  double *R = d.red + (long long)g * RG_NRED;
  const double tol = R[R_TOL];
  const int imax = (int)R[R_IMAX];
  for (int c = 0; c < 2; ++c) {
    if (R[R_ACTIVE + c] != 0.0) {
      const double rho = R[R_ACC1 + c];
      R[R_BETA + c] = rho / R[R_RHO + c];
      R[R_RHO + c] = rho;
      const double it = R[R_ITERS + c] + 1.0;
      R[R_ITERS + c] = it;
      R[R_ACTIVE + c] = (it < imax && sqrt(rho) / R[R_BNORM + c] > tol) ? 1.0 : 0.0;
    }
    R[R_ACC0 + c] = 0.0;
    R[R_ACC1 + c] = 0.0;
  }
  if (R[R_ACTIVE] != 0.0 || R[R_ACTIVE + 1] != 0.0) atomicAdd(d.n_active, 1);
}

__global__ void k_qeq_sums(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[2] = {0, 0};
  if (s < d.n) {
    const double2 x = d.qx[s];
    v[0] = x.x;
    v[1] = x.y;
  }
  seg_block_add<2>(v, seg_at(d, s), d.red + R_SUM, RG_NRED);
}

// q = s - (sum s / sum t) t per segment; shift histories (original order)
__global__ void k_qeq_finish(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.n) return;
  const int n = d.n, i = d.perm[s];
  const double *R = d.red + (long long)d.seg_s[s] * RG_NRED;
  const double u = R[R_SUM] / R[R_SUM + 1];
  const double2 x = d.qx[s];
  const double q = x.x - u * x.y;
  d.q_o[i] = q;
  d.xs[s].w = q;
  const float qh = __double2float_rn(q);
  d.xl[s].w = qh;
  d.qlo[s] = __double2float_rn(q - (double)qh);
  for (int k = 4; k > 0; --k) {
    d.s_hist[k * n + i] = d.s_hist[(k - 1) * n + i];
    d.t_hist[k * n + i] = d.t_hist[(k - 1) * n + i];
  }
  d.s_hist[i] = x.x;
  d.t_hist[i] = x.y;
}

}  // namespace

void launch_qeq_setup(const Dev &d, cudaStream_t st) {
  const int B = 256;
  k_qeq_setup<<<(d.n + B - 1) / B, B, 0, st>>>(d);
}

// the row-group width (lanes per row) chosen by the autotuner, d.spmv_rw
template <int RW>
static void spmv_rw(const Dev &d, cudaStream_t st, const double2 *x, double2 *y, int use_act,
                    int kind) {
  const unsigned G = (unsigned)(((long long)d.n * RW + 255) / 256);
  if (kind == 0) k_spmvp<RW><<<G, 256, 0, st>>>(d, x, y, use_act);
  else k_spmv32<RW><<<G, 256, 0, st>>>(d, x, y, use_act);
}

static void spmv_kind(const Dev &d, cudaStream_t st, const double2 *x, double2 *y, int use_act,
                      int kind) {
  if (d.spmv_rw == 8) spmv_rw<8>(d, st, x, y, use_act, kind);
  else if (d.spmv_rw == 32) spmv_rw<32>(d, st, x, y, use_act, kind);
  else spmv_rw<16>(d, st, x, y, use_act, kind);
}

// the compensated SpMV of the split copy of x in qd32 (of qd after the
// kernels that update it), with the FP64 form's FP32-pair H or the mixed
// form's FP32 H
void launch_qeq_spmv(const Dev &d, cudaStream_t st, const double2 *x, double2 *y, int use_act) {
  spmv_kind(d, st, x, y, use_act, d.mixed ? 1 : 0);
}

// the split FP32 pair copy of x that k_spmv32 reads
__global__ void k_split_x(Dev d, const double2 *__restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.n) d.qd32[i] = split4(x[i]);
}

// r = b - H x of the current iterate starts the CG (the SpMV of the
// iterations, on the split copy of x); the mixed form's restarts come from
// launch_qeq_refine_check + launch_qeq_cg_init_rest.
void launch_qeq_cg_init(const Dev &d, cudaStream_t st, double tol, int imax) {
  const int B = 256, G = (d.n + B - 1) / B;
  k_split_x<<<G, B, 0, st>>>(d, d.qx);
  launch_qeq_spmv(d, st, d.qx, d.qq, 0);
  k_cg_init1<<<G, B, 0, st>>>(d);
  launch_qeq_cg_init_rest(d, st, tol, imax);
}

// The mixed form's refinement check: b.b and u.r of the true residual
// r = b - H x (the compensated SpMV of the split iterate: products exact,
// sums to ~1e-13 of |H||x|, far below the 1e-6 tolerance, where the CG's
// recurrence residual has drifted) and u = r Hdia_inv per segment; a
// segment needs a restart only where sqrt(u.r) / |b| is above the
// tolerance (the criterion of k_cg_init_ctrl), and the rest of the set-up
// runs only then.
__global__ void k_refine_sums(Dev d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (s < d.n) {
    const double2 u = d.qu[s], r = d.qr[s], b = d.qb[s];
    v[0] = b.x * b.x; v[1] = b.y * b.y;
    v[2] = u.x * r.x; v[3] = u.y * r.y;
  }
  seg_block_add<4>(v, seg_at(d, s), d.red + R_INIT, RG_NRED);
}

__global__ void k_refine_ctrl(Dev d, double tol) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nseg) return;
  const double *R = d.red + (long long)g * RG_NRED;
  bool need = false;
  for (int c = 0; c < 2; ++c)
    need = need || sqrt(R[R_INIT + 2 + c]) / sqrt(R[R_INIT + c]) > tol;
  if (need) atomicAdd(d.n_active, 1);
}

void launch_qeq_refine_check(const Dev &d, cudaStream_t st, double tol) {
  const int B = 256, G = (d.n + B - 1) / B;
  const int GS = (d.nseg + 127) / 128;
  k_split_x<<<G, B, 0, st>>>(d, d.qx);
  spmv_kind(d, st, d.qx, d.qq, 0, 1);
  k_cg_init1<<<G, B, 0, st>>>(d);
  k_seg_zero<<<GS, 128, 0, st>>>(d, R_INIT, 4);
  k_refine_sums<<<G, B, 0, st>>>(d);
  cudaMemsetAsync(d.n_active, 0, sizeof(int), st);
  k_refine_ctrl<<<GS, 128, 0, st>>>(d, tol);
}

// the set-up after r and u (k_cg_init1, which also set p = u): the CG
// scalars
void launch_qeq_cg_init_rest(const Dev &d, cudaStream_t st, double tol, int imax) {
  const int B = 256, G = (d.n + B - 1) / B;
  const int GS = (d.nseg + 127) / 128;
  k_seg_zero<<<GS, 128, 0, st>>>(d, R_INIT, 4);
  k_cg_init_sums<<<G, B, 0, st>>>(d);
  cudaMemsetAsync(d.n_active, 0, sizeof(int), st);
  k_cg_init_ctrl<<<GS, 128, 0, st>>>(d, tol, imax);
}

// one CG iteration = launch_qeq_cg_A (p), SpMV of p into q,
// launch_qeq_cg_C (p.q, the updates and u.r, the control)
void launch_qeq_cg_A(const Dev &d, cudaStream_t st) {
  const int B = 256, G = (d.n + B - 1) / B;
  k_pcg_p<<<G, B, 0, st>>>(d);
}

void launch_qeq_cg_C(const Dev &d, cudaStream_t st) {
  const int B = 256, G = (d.n + B - 1) / B;
  const int GS = (d.nseg + 127) / 128;
  if (d.nseg == 1) {
    const int G1 = G < 608 ? G : 608;
    k_pcg_sigma<true><<<G1, B, 0, st>>>(d);
    k_pcg_update<true><<<G1, B, 0, st>>>(d);
  } else {
    k_pcg_sigma<false><<<G, B, 0, st>>>(d);
    k_pcg_update<false><<<G, B, 0, st>>>(d);
  }
  k_pcg_ctrl<<<GS, 128, 0, st>>>(d);
}

void launch_qeq_finish(const Dev &d, cudaStream_t st) {
  const int B = 256, G = (d.n + B - 1) / B;
  k_seg_zero<<<(d.nseg + 127) / 128, 128, 0, st>>>(d, R_SUM, 2);
  k_qeq_sums<<<G, B, 0, st>>>(d);
  k_qeq_finish<<<G, B, 0, st>>>(d);
}

// ------------------------------------------------------------------
// QEq control of the captured step (conditional graph nodes)

namespace {

__global__ void k_set_cond(const int *n_active, cudaGraphConditionalHandle c1,
                           cudaGraphConditionalHandle c2, int two) {
  const unsigned v = *n_active > 0 ? 1u : 0u;
  cudaGraphSetConditional(c1, v);
  if (two) cudaGraphSetConditional(c2, v);
}

// after one CG iteration (k_cg_flip has recounted the active segments); the
// trip limit bounds the loop even if the per-segment iteration limit failed
__global__ void k_loop_cond(const int *n_active, int *ctl, cudaGraphConditionalHandle c,
                            int limit) {
  const int trips = ++ctl[1];
  unsigned v = *n_active > 0 ? 1u : 0u;
  if (v && trips >= limit) {
    ctl[2] = 1;
    v = 0u;
  }
  cudaGraphSetConditional(c, v);
}

__global__ void k_qeq_tot(Dev d, int pass) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nseg) return;
  const double *R = d.red + (long long)g * RG_NRED;
  for (int c = 0; c < 2; ++c) {
    const int it = (int)R[R_ITERS + c] - (pass ? 1 : 0);
    d.qeq_tot[2 * g + c] += it > 0 ? it : 0;
  }
}

__global__ void k_restart_count(int *ctl) { ++ctl[0]; }

}  // namespace

void launch_qeq_set_cond(const Dev &d, cudaStream_t st, unsigned long long c1,
                         unsigned long long c2) {
  k_set_cond<<<1, 1, 0, st>>>(d.n_active, (cudaGraphConditionalHandle)c1,
                              (cudaGraphConditionalHandle)c2, c2 != 0);
}

void launch_qeq_loop_cond(const Dev &d, cudaStream_t st, unsigned long long c, int limit) {
  k_loop_cond<<<1, 1, 0, st>>>(d.n_active, d.qeq_ctl, (cudaGraphConditionalHandle)c, limit);
}

void launch_qeq_tot(const Dev &d, cudaStream_t st, int pass) {
  k_qeq_tot<<<(d.nseg + 127) / 128, 128, 0, st>>>(d, pass);
}

void launch_qeq_restart_count(const Dev &d, cudaStream_t st) {
  k_restart_count<<<1, 1, 0, st>>>(d.qeq_ctl);
}
