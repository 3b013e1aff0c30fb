// Velocity-Verlet NVE integration (fix nve/sunway): the two half steps of
// fix_nve_sw64.c:25-172 with dtf = 0.5 dt ftm2v (fix_nve_sunway.cpp:54-58),
// per-type masses (the force field's unless the caller set the data
// file's, rg_set_masses).  Arrays are in the original order.
#include "rg_internal.h"

namespace {

// LAMMPS real units: ftm2v = 1 / 48.88821291^2
constexpr double FTM2V = 1.0 / 48.88821291 / 48.88821291;

__global__ void k_nve_initial(Dev d, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const double dtf = 0.5 * dt * FTM2V;
  const double dtfm = dtf / d.ff->nve_mass[d.type_o[i]];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double v = d.v_o[3 * i + c] + dtfm * d.f_o[3 * i + c];
    d.v_o[3 * i + c] = v;
    d.x_o[3 * i + c] += dt * v;
  }
}

__global__ void k_nve_final(Dev d, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const double dtf = 0.5 * dt * FTM2V;
  const double dtfm = dtf / d.ff->nve_mass[d.type_o[i]];
#pragma unroll
  for (int c = 0; c < 3; ++c) d.v_o[3 * i + c] += dtfm * d.f_o[3 * i + c];
}

}  // namespace

void launch_nve_initial(const Dev &d, cudaStream_t st, double dt) {
  k_nve_initial<<<(d.n + 255) / 256, 256, 0, st>>>(d, dt);
}

void launch_nve_final(const Dev &d, cudaStream_t st, double dt) {
  k_nve_final<<<(d.n + 255) / 256, 256, 0, st>>>(d, dt);
}
