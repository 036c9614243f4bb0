// Fused Langevin integrator kernels (compiled with --fmad=false).
//
// The reference launches one kernel per phase (11 phase launches plus the
// post-step clamp and RATTLE, fused_engine.rs:19268-19455, :17498-17800)
// because its per-atom and per-cluster phases index different thread spaces.
// Here a thread owns a whole constraint unit, so all phases between two force
// evaluations run in one launch: post(s-1) followed by pre(s).
#include "pq_phases.cuh"

namespace pq {

// Six resident blocks per SM (80 registers) trade a few spilled words for
// twice the occupancy of the unconstrained 112-register build.
__global__ void __launch_bounds__(128, 6) k_integrate(Arena A, int64_t n_units, int mode) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_units) return;
  const Unit U = A.units[t];
  if (U.nh < 0) return;
  SysDev* Sp = &A.sys[U.sys];
  const SysDev S = *Sp;
  if (!S.active || S.status != 0) return;
  const long long s = S.step;
  const bool com_step = S.com_interval > 0 && s > 0 && (s % S.com_interval) == 0;
  UnitState u;
  int local[4];
  load_unit(A, U, u, local, S.atom_begin);
  int err = 0;
  if ((mode & kIntPost) && s > 0) err = phases_post(u, U, S, local, (uint64_t)(s - 1));
  // On a COM step the pre-phase waits for the per-system COM reduction,
  // which runs in the control kernel.
  if (!err && (mode & kIntPre) && !com_step) {
    err = phases_pre(u, U, S, local, (uint64_t)s);
    if (!err) check_displacement(A, U, u, Sp);
  }
  if (!err && !unit_finite(u)) err = kStNonfinite;
  if (err) {
    atomicOr(&Sp->status, err);
    return;
  }
  store_unit(A, U, u);
}

// Single phase sets for the parity tests; `step` selects the noise.
__global__ void __launch_bounds__(128) k_debug_phases(Arena A, int64_t n_units, int set,
                                                      long long step) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_units) return;
  const Unit U = A.units[t];
  if (U.nh < 0) return;
  SysDev* Sp = &A.sys[U.sys];
  const SysDev S = *Sp;
  if (!S.active) return;
  UnitState u;
  int local[4];
  load_unit(A, U, u, local, S.atom_begin);
  int err = set == kIntPre ? phases_pre(u, U, S, local, (uint64_t)step)
                           : phases_post(u, U, S, local, (uint64_t)step);
  if (err) atomicOr(&Sp->status, err);
  store_unit(A, U, u);
}

// Per-system energy totals in a fixed reduction order: out[6*s + c] for the
// five potential planes and the kinetic energy.
__global__ void __launch_bounds__(256) k_energy_reduce(Arena A, double* out) {
  const int s = blockIdx.x;
  const SysDev S = A.sys[s];
  __shared__ double red[6][256];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  if (S.active) {
    for (int i = threadIdx.x; i < S.n_atoms; i += blockDim.x) {
      const int a = S.atom_begin + i;
      for (int c = 0; c < 5; ++c) acc[c] += A.pe[(int64_t)c * A.atom_cap + a];
      const float4 v = A.vel[a];
      const double v2 = (double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z;
      acc[5] += 0.5 * (double)v.w * v2 / (double)kKcalToAmuA2Ps2;
    }
  }
  for (int c = 0; c < 6; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 6; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 6) out[6 * s + threadIdx.x] = red[threadIdx.x][0];
}

void launch_integrate(const Arena& A, int64_t n_units_span, int mode, cudaStream_t st) {
  if (n_units_span <= 0) return;
  const int64_t blocks = (n_units_span + 127) / 128;
  k_integrate<<<(unsigned)blocks, 128, 0, st>>>(A, n_units_span, mode);
}

void launch_debug_phases(const Arena& A, int64_t n_units_span, int set, long long step,
                         cudaStream_t st) {
  if (n_units_span <= 0) return;
  const int64_t blocks = (n_units_span + 127) / 128;
  k_debug_phases<<<(unsigned)blocks, 128, 0, st>>>(A, n_units_span, set, step);
}

void launch_energy_reduce(const Arena& A, int n_sys, double* out6, cudaStream_t st) {
  if (n_sys <= 0) return;
  k_energy_reduce<<<n_sys, 256, 0, st>>>(A, out6);
}

}  // namespace pq
