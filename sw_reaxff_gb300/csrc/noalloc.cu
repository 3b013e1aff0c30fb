// rg_qeq_noalloc: QEq charges without any device allocation at call time.
//
// For callers that cannot call cudaMalloc when they need charges: code that
// runs under a host application's own device-memory manager (which forbids
// or does not see allocations made behind its back), or inside a region
// where a device allocation would synchronize or fail.  The caller owns the
// input and output device arrays; the QEq matrix H is evaluated on the fly
// (never stored) and the CG work vectors live in one static device array of
// fixed size, RG_NOALLOC_MAX_ATOMS atoms.  Positions may lie outside the
// box: the first kernel wraps them into [0, L) (in the scratch array), as
// rg_set_atoms does for the main path.
//
// The scratch array is shared by every call on a device and keeps the
// previous call's contents; each call clears what it needs.  Calls whose
// GPU work overlaps (different streams, or host threads) race on it.
//
// The mathematics is that of rg_qeq's first solve after rg_set_atoms (zero
// initial guesses): dual pipelined Jacobi-PCG of CG_v2
// (fix_qeq_reax_sunway.cpp:983-1167) and calculate_Q (:1697-1755).
#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/reaxgpu.h"
#include "rg_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NMAX = RG_NOALLOC_MAX_ATOMS;
// 12 double2 vectors + Jacobi diagonal + 128 scalars + wrapped positions
constexpr size_t NA_DOUBLES = 24 * (size_t)NMAX + NMAX + 128 + 3 * (size_t)NMAX;

__device__ __align__(256) double rg_noalloc_scratch[NA_DOUBLES];

// scalar slots (pairs [s, t]) in the last 128 doubles
enum {
  S_ACC0 = 0, S_ACC1 = 2, S_ALPHA = 6, S_ALPHA_OLD = 8, S_BETA = 10, S_SIG = 12,
  S_HETA = 14, S_BNORM = 16, S_ACTIVE = 20, S_ITERS = 22, S_SUM = 24, S_BAD = 26,
  S_INIT = 32, S_NEXT = 52
};

struct View {
  int n;
  double2 *x, *b, *r, *u, *w, *d, *q, *p, *s, *v, *z, *m;
  double *hdi, *R, *xw;
};

View make_view(double *base, int n) {
  View V;
  V.n = n;
  double2 *vec = reinterpret_cast<double2 *>(base);
  double2 **slots[12] = {&V.x, &V.b, &V.r, &V.u, &V.w, &V.d, &V.q, &V.p, &V.s, &V.v, &V.z, &V.m};
  for (int k = 0; k < 12; ++k) *slots[k] = vec + (size_t)k * NMAX;
  V.hdi = base + 24 * (size_t)NMAX;
  V.R = base + 25 * (size_t)NMAX;
  V.xw = V.R + 128;
  return V;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
  return v;
}

template <int K>
__device__ __forceinline__ void block_add_k(double *v, double *dst) {
  __shared__ double red[K][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < K; ++c) v[c] = warp_sum(v[c]);
  if (l == 0)
#pragma unroll
    for (int c = 0; c < K; ++c) red[c][w] = v[c];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int c = 0; c < K; ++c) {
      double x = (l < (int)(blockDim.x >> 5)) ? red[c][l] : 0.0;
      x = warp_sum(x);
      if (l == 0) atomicAdd(&dst[c], x);
    }
  }
}

struct Geo {
  const double *x;
  const int *type;
  double L[3];
  int k[3];          // image range per dimension
};

// x - L floor(x / L), rounded per operation like the main path's binning
__device__ __forceinline__ double na_wrap(double x, double L) {
  double y = __dsub_rn(x, __dmul_rn(L, floor(__ddiv_rn(x, L))));
  if (y >= L) y = __dsub_rn(y, L);
  if (y < 0.0) y = 0.0;
  return y;
}

// Jacobi diagonal, right-hand sides, zero guesses, wrapped positions; a
// non-finite position or a type outside the force field sets R[S_BAD] and
// leaves the atom out (the host then rejects the call)
__global__ void k_na_setup(View V, Geo G, const ForceField *ff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  const int ti = G.type[i];
  const double x0 = G.x[3 * i], y0 = G.x[3 * i + 1], z0 = G.x[3 * i + 2];
  const bool ok = ti >= 0 && ti < ff->ntypes && isfinite(x0) && isfinite(y0) && isfinite(z0);
  if (!ok) {
    V.R[S_BAD] = 1.0;
    V.hdi[i] = 0.0;
    V.b[i] = make_double2(0.0, 0.0);
    V.x[i] = make_double2(0.0, 0.0);
    V.xw[3 * i] = V.xw[3 * i + 1] = V.xw[3 * i + 2] = 0.0;
    return;
  }
  V.xw[3 * i] = na_wrap(x0, G.L[0]);
  V.xw[3 * i + 1] = na_wrap(y0, G.L[1]);
  V.xw[3 * i + 2] = na_wrap(z0, G.L[2]);
  const Sbp &sb = ff->sbp[ti];
  V.hdi[i] = 1. / sb.eta;
  V.b[i] = make_double2(-sb.chi, -1.0);
  V.x[i] = make_double2(0.0, 0.0);
}

// y = (eta + H) x with H evaluated on the fly; one warp per row
__global__ void __launch_bounds__(256) k_na_matvec(View V, Geo G, const ForceField *ff,
                                                   const Control *ctl, const double2 *in,
                                                   double2 *out) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= V.n) return;
  const double xi = V.xw[3 * i], yi = V.xw[3 * i + 1], zi = V.xw[3 * i + 2];
  const int ti = G.type[i];
  const double swb2 = ctl->swb2;
  const double *T = ctl->qTap;
  double as = 0.0, at = 0.0;
  for (int j = lane; j < V.n; j += 32) {
    const double xj = V.xw[3 * j], yj = V.xw[3 * j + 1], zj = V.xw[3 * j + 2];
    const double shld = ff->tbp[ti][G.type[j]].gamma;
    const double2 vj = in[j];
    for (int sz = -G.k[2]; sz <= G.k[2]; ++sz)
      for (int sy = -G.k[1]; sy <= G.k[1]; ++sy)
        for (int sx = -G.k[0]; sx <= G.k[0]; ++sx) {
          if (j == i && sx == 0 && sy == 0 && sz == 0) continue;
          const double dx = __dsub_rn(__dadd_rn(xj, sx * G.L[0]), xi);
          const double dy = __dsub_rn(__dadd_rn(yj, sy * G.L[1]), yi);
          const double dz = __dsub_rn(__dadd_rn(zj, sz * G.L[2]), zi);
          const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
          if (d2 > swb2) continue;
          const double r = __dsqrt_rn(d2);
          double tp = fma(T[7], r, T[6]);
          tp = fma(tp, r, T[5]);
          tp = fma(tp, r, T[4]);
          tp = fma(tp, r, T[3]);
          tp = fma(tp, r, T[2]);
          tp = fma(tp, r, T[1]);
          tp = fma(tp, r, T[0]);
          const double h = tp * 14.4 / pow_third(r * r * r + shld, RG_C3_QEQ);
          as = fma(h, vj.x, as);
          at = fma(h, vj.y, at);
        }
  }
  as = warp_sum(as);
  at = warp_sum(at);
  if (lane == 0) {
    const double eta = ff->sbp[ti].eta;
    const double2 v = in[i];
    out[i] = make_double2(fma(eta, v.x, as), fma(eta, v.y, at));
  }
}

__global__ void k_na_init1(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  const double hi = V.hdi[i];
  const double2 b = V.b[i], q = V.q[i];
  const double2 r = make_double2(b.x - q.x, b.y - q.y);
  V.r[i] = r;
  V.u[i] = make_double2(r.x * hi, r.y * hi);
  V.d[i] = V.u[i];
}

__global__ void k_na_init2(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  const double hi = V.hdi[i];
  const double2 q = V.q[i];
  V.w[i] = q;
  V.m[i] = make_double2(q.x * hi, q.y * hi);
  V.d[i] = V.m[i];
}

__global__ void k_na_init3(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (i < V.n) {
    const double2 u = V.u[i], w = V.w[i], m = V.m[i], r = V.r[i], b = V.b[i];
    V.p[i] = u;
    V.s[i] = w;
    V.v[i] = m;
    V.z[i] = V.q[i];
    a[0] = b.x * b.x; a[1] = b.y * b.y;
    a[2] = u.x * r.x; a[3] = u.y * r.y;
    a[4] = u.x * w.x; a[5] = u.y * w.y;
  }
  block_add_k<6>(a, V.R + S_INIT);
}

__global__ void k_na_init_ctrl(View V, double tol, int imax) {
  double *R = V.R;
  for (int c = 0; c < 2; ++c) {
    const double bb = R[S_INIT + c], ur = R[S_INIT + 2 + c], uw = R[S_INIT + 4 + c];
    R[S_BNORM + c] = sqrt(bb);
    R[S_SIG + c] = ur;
    R[S_HETA + c] = uw;
    R[S_ALPHA + c] = ur / uw;
    R[S_ITERS + c] = 1.0;
    R[S_ACTIVE + c] = (1 < imax && sqrt(ur) / R[S_BNORM + c] > tol) ? 1.0 : 0.0;
    R[S_ACC0 + c] = 0.0;
    R[S_ACC1 + c] = 0.0;
  }
}

__global__ void k_na_A(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double *R = V.R;
  const bool as = R[S_ACTIVE] != 0.0, at = R[S_ACTIVE + 1] != 0.0;
  double a[4] = {0, 0, 0, 0};
  if (i < V.n && (as || at)) {
    const double hi = V.hdi[i];
    double2 r = V.r[i], u = V.u[i], w = V.w[i], dd = V.d[i];
    const double2 s = V.s[i], v = V.v[i], z = V.z[i];
    if (as) {
      const double al = R[S_ALPHA];
      r.x -= al * s.x; u.x -= al * v.x; w.x -= al * z.x;
      a[0] = u.x * r.x; a[2] = u.x * w.x;
      dd.x = w.x * hi;
    }
    if (at) {
      const double al = R[S_ALPHA + 1];
      r.y -= al * s.y; u.y -= al * v.y; w.y -= al * z.y;
      a[1] = u.y * r.y; a[3] = u.y * w.y;
      dd.y = w.y * hi;
    }
    V.r[i] = r; V.u[i] = u; V.w[i] = w; V.d[i] = dd;
  }
  block_add_k<4>(a, V.R + S_ACC0);
}

__global__ void k_na_ctrl(View V, double tol, int imax) {
  double *R = V.R;
  for (int c = 0; c < 2; ++c) {
    if (R[S_ACTIVE + c] == 0.0) {
      R[S_ACC0 + c] = 0.0;
      R[S_ACC1 + c] = 0.0;
      continue;
    }
    const double dot0 = R[S_ACC0 + c], dot1 = R[S_ACC1 + c];
    const double beta = dot0 / R[S_SIG + c];
    const double heta = dot1 - beta * beta * R[S_HETA + c];
    R[S_BETA + c] = beta;
    R[S_HETA + c] = heta;
    R[S_ALPHA_OLD + c] = R[S_ALPHA + c];
    R[S_ALPHA + c] = dot0 / heta;
    R[S_SIG + c] = dot0;
    R[S_ACC0 + c] = 0.0;
    R[S_ACC1 + c] = 0.0;
    const double it = R[S_ITERS + c] + 1.0;
    R[S_ITERS + c] = it;
    R[S_NEXT + c] = (it < imax && sqrt(dot0) / R[S_BNORM + c] > tol) ? 1.0 : 0.0;
  }
}

__global__ void k_na_C(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double *R = V.R;
  const bool as = R[S_ACTIVE] != 0.0, at = R[S_ACTIVE + 1] != 0.0;
  if (i >= V.n || !(as || at)) return;
  double2 x = V.x[i], p = V.p[i], s = V.s[i], v = V.v[i], z = V.z[i];
  const double2 u = V.u[i], w = V.w[i], dd = V.d[i], q = V.q[i];
  if (as) {
    const double al = R[S_ALPHA_OLD], be = R[S_BETA];
    x.x += al * p.x; p.x = u.x + p.x * be; s.x = w.x + s.x * be; v.x = dd.x + v.x * be; z.x = q.x + z.x * be;
  }
  if (at) {
    const double al = R[S_ALPHA_OLD + 1], be = R[S_BETA + 1];
    x.y += al * p.y; p.y = u.y + p.y * be; s.y = w.y + s.y * be; v.y = dd.y + v.y * be; z.y = q.y + z.y * be;
  }
  V.x[i] = x; V.p[i] = p; V.s[i] = s; V.v[i] = v; V.z[i] = z;
}

__global__ void k_na_flip(View V) {
  double *R = V.R;
  for (int c = 0; c < 2; ++c)
    if (R[S_ACTIVE + c] != 0.0) R[S_ACTIVE + c] = R[S_NEXT + c];
}

__global__ void k_na_sums(View V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[2] = {0, 0};
  if (i < V.n) {
    a[0] = V.x[i].x;
    a[1] = V.x[i].y;
  }
  block_add_k<2>(a, V.R + S_SUM);
}

__global__ void k_na_finish(View V, double *q_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  const double u = V.R[S_SUM] / V.R[S_SUM + 1];
  q_out[i] = V.x[i].x - u * V.x[i].y;
}

// per-device address of the scratch array (set once per device)
double *g_scratch[64] = {nullptr};

// restores the caller's current device on every return
struct DeviceRestore {
  int prev = -1;
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int na_fail(rg_system *h, int code, const std::string &msg) {
  rg_set_error(h, "rg_qeq_noalloc: " + msg);
  return code;
}

int na_cuda(rg_system *h, cudaError_t e, const char *what) {
  return na_fail(h, RG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

// The handle supplies only the force-field and control tables it copied to
// the device at rg_create; nothing of it is written here.
extern "C" int rg_qeq_noalloc(rg_system *h, int n, const double *x, const int *type,
                              const double *box3, double *q_out, int *iters_s, int *iters_t,
                              void *stream) {
  if (!h) return RG_E_ARG;
  if (!x || !type || !box3 || !q_out)
    return na_fail(h, RG_E_ARG, "x, type, box3 and q_out must not be NULL");
  if (n < 1 || n > NMAX)
    return na_fail(h, RG_E_ARG, "n must be in [1, " + std::to_string(NMAX) +
                                    "] (static scratch size), got " + std::to_string(n));
  const ForceField *ff = nullptr;
  const Control *ctl = nullptr;
  int device = 0;
  double swb = 0, tol = 0;
  int imax = 0;
  rg_noalloc_tables(h, &ff, &ctl, &device, &swb, &tol, &imax);
  if (device < 0 || device >= 64)
    return na_fail(h, RG_E_ARG, "device index " + std::to_string(device) + " outside [0, 64)");
  Geo G;
  G.x = x;
  G.type = type;
  for (int k = 0; k < 3; ++k) {
    // the main path's limit: no edge shorter than half the cutoff, which
    // also bounds the image range below at ceil(swb / L) <= 2
    if (!std::isfinite(box3[k]) || !(box3[k] >= 0.5 * swb))
      return na_fail(h, RG_E_ARG, "box edges must be finite and at least half the QEq cutoff (" +
                                      std::to_string(0.5 * swb) + " A)");
    G.L[k] = box3[k];
    G.k[k] = (int)std::ceil(swb / box3[k]);
  }
  DeviceRestore restore;
  cudaError_t e = cudaGetDevice(&restore.prev);
  if (e != cudaSuccess) return na_cuda(h, e, "cudaGetDevice");
  if ((e = cudaSetDevice(device)) != cudaSuccess) return na_cuda(h, e, "cudaSetDevice");
  if (!g_scratch[device]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, rg_noalloc_scratch);
    if (e != cudaSuccess || !p) return na_cuda(h, e, "cudaGetSymbolAddress");
    g_scratch[device] = (double *)p;
  }
  cudaStream_t st = (cudaStream_t)stream;
  View V = make_view(g_scratch[device], n);
  // scalars start from zero on every call
  if ((e = cudaMemsetAsync(V.R, 0, 128 * sizeof(double), st)) != cudaSuccess)
    return na_cuda(h, e, "cudaMemsetAsync");
  const int B = 256, Gr = (n + B - 1) / B;
  const unsigned Gw = (unsigned)(((long long)n * 32 + 255) / 256);
  k_na_setup<<<Gr, B, 0, st>>>(V, G, ff);
  // the products index the parameter tables by every partner's type: check
  // the inputs before the first one
  double bad = 0.0;
  if ((e = cudaMemcpyAsync(&bad, V.R + S_BAD, sizeof(double), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return na_cuda(h, e, "input check");
  if (bad != 0.0)
    return na_fail(h, RG_E_ARG, "a position is not finite or a type is outside the force field");
  k_na_matvec<<<Gw, 256, 0, st>>>(V, G, ff, ctl, V.x, V.q);
  k_na_init1<<<Gr, B, 0, st>>>(V);
  k_na_matvec<<<Gw, 256, 0, st>>>(V, G, ff, ctl, V.d, V.q);
  k_na_init2<<<Gr, B, 0, st>>>(V);
  k_na_matvec<<<Gw, 256, 0, st>>>(V, G, ff, ctl, V.d, V.q);
  k_na_init3<<<Gr, B, 0, st>>>(V);
  k_na_init_ctrl<<<1, 1, 0, st>>>(V, tol, imax);
  double flags[4];
  int done = 0;
  for (;;) {
    if ((e = cudaMemcpyAsync(flags, V.R + S_ACTIVE, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return na_cuda(h, e, "CG control read");
    if (flags[0] == 0.0 && flags[1] == 0.0) break;
    if (done > imax + 8) return na_fail(h, RG_E_NUMERIC, "iteration control lost");
    for (int k = 0; k < 4; ++k) {
      k_na_A<<<Gr, B, 0, st>>>(V);
      k_na_matvec<<<Gw, 256, 0, st>>>(V, G, ff, ctl, V.d, V.q);
      k_na_ctrl<<<1, 1, 0, st>>>(V, tol, imax);
      k_na_C<<<Gr, B, 0, st>>>(V);
      k_na_flip<<<1, 1, 0, st>>>(V);
    }
    done += 4;
  }
  k_na_sums<<<Gr, B, 0, st>>>(V);
  k_na_finish<<<Gr, B, 0, st>>>(V, q_out);
  if ((e = cudaGetLastError()) != cudaSuccess) return na_cuda(h, e, "kernel launch");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return na_cuda(h, e, "final sync");
  if (iters_s) *iters_s = (int)flags[2];
  if (iters_t) *iters_t = (int)flags[3];
  return RG_OK;
}
