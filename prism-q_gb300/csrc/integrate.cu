// Fused Langevin integrator kernels (compiled with --fmad=false).
//
// The reference launches one kernel per phase (11 phase launches plus the
// post-step clamp and RATTLE, fused_engine.rs:19268-19455, :17498-17800)
// because its per-atom and per-cluster phases index different thread spaces.
// Here a thread owns a whole constraint unit, so all phases between two force
// evaluations run in one launch: post(s-1) followed by pre(s).
#include "pq_phases.cuh"

namespace pq {

// One thread per constraint unit.  The OU normals arrive drawn (k_noise), and
// six resident blocks per SM (80 registers, a few spilled words) are the
// measured balance between occupancy and spills: on the 256-system workload
// the launch takes 0.074 ms against 0.086 ms at eight blocks (64 registers)
// and 0.085 ms at four (102 registers, no spills).
// R = float: the production step, for the systems whose constraint checks run
// in FP32 (kCheck64 false) or FP64 (kCheck64 true); R = double: the
// FP64-everywhere step of an FP64 batch.
// The grid walks the batch-wide unit order (n_units entries: the ranges of
// A.order_range), so the units with the longest constraint chains are
// scheduled first.
__device__ __forceinline__ int ordered_unit(const Arena& A, int t) {
  // the last range whose first walk position is <= t (it is never empty)
  int lo = 0, hi = A.n_ranges - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(A.order_prefix + mid) <= t) lo = mid;
    else hi = mid - 1;
  }
  return __ldg(&A.order_range[lo].x) + (t - __ldg(A.order_prefix + lo));
}

template <class R, bool kCheck64>
__global__ void __launch_bounds__(128, 6) k_integrate(Arena A, int64_t n_units, int mode) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_units) return;
  const Unit U = A.units[ordered_unit(A, (int)t)];
  if (U.nh < 0) return;
  SysDev* Sp = &A.sys[U.sys];
  const SysDev S = *Sp;
  if (!S.active || S.status != 0) return;
  if (sizeof(R) == 4 && (S.check64 != 0) != kCheck64) return;
  const long long s = S.step;
  const bool com_step = S.com_interval > 0 && s > 0 && (s % S.com_interval) == 0;
  UnitStateT<R> u;
  int local[4];
  load_unit(A, U, u, local, S.atom_begin);
  int err = 0;
  if ((mode & kIntPost) && s > 0) {
    SysDev SP = S;  // the post-force phases run with their own step's parameters
    SP.dt = S.post_dt;
    SP.temperature = S.post_temperature;
    SP.gamma = S.post_gamma;
    SP.c1 = S.post_c1;
    SP.c1d = S.post_c1d;
    err = phases_post<R, kCheck64, true>(u, U, SP, local, (uint64_t)(s - 1), A.noise);
  }
  // On a COM step the pre-phase waits for the per-system COM reduction,
  // which runs in the control kernel.
  const bool pre = (mode & kIntPre) && !com_step;
  if (!err && pre) {
    err = phases_pre<R, kCheck64, true>(u, U, S, local, (uint64_t)s, A.noise + A.atom_cap);
    if (!err) check_displacement(A, U, u, Sp);
  }
  if (!err && !unit_finite(u)) err = kStNonfinite;
  if (err) {
    atomicOr(&Sp->status, err);
    return;
  }
  store_unit(A, U, u, pre);
}

// The OU normals of the next integrate launch, one thread per atom.  Drawing
// them here, with every atom in flight at once, takes the Philox rounds and
// the Box–Muller series out of the integrator's per-unit dependency chains;
// the values are the ones normal3 gives there, bit for bit.
__global__ void __launch_bounds__(256) k_noise(Arena A, int64_t n_atoms, int mode) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_atoms) return;
  const int sid = A.atom_sys[a];
  if (sid < 0) return;
  const SysDev& S = A.sys[sid];
  if (!S.active || S.status != 0) return;
  const long long s = S.step;
  const uint32_t local = (uint32_t)(a - S.atom_begin);
  float z0, z1, z2;
  if ((mode & kIntPost) && s > 0 && S.post_gamma != 0.0f) {
    normal3(S.seed, S.stream, local, (uint64_t)(s - 1), kPurposeOuNp1, &z0, &z1, &z2);
    A.noise[a] = make_float4(z0, z1, z2, 0.0f);
  }
  const bool com_step = S.com_interval > 0 && s > 0 && (s % S.com_interval) == 0;
  if ((mode & kIntPre) && !com_step && S.gamma != 0.0f) {
    normal3(S.seed, S.stream, local, (uint64_t)s, kPurposeOuN, &z0, &z1, &z2);
    A.noise[A.atom_cap + a] = make_float4(z0, z1, z2, 0.0f);
  }
}

void launch_noise(const Arena& A, int64_t n_atoms_span, int mode, cudaStream_t st) {
  if (n_atoms_span <= 0) return;
  k_noise<<<(unsigned)((n_atoms_span + 255) / 256), 256, 0, st>>>(A, n_atoms_span, mode);
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
  int err = set == kIntPre ? phases_pre<float, false>(u, U, S, local, (uint64_t)step)
                           : phases_post<float, false>(u, U, S, local, (uint64_t)step);
  if (err) atomicOr(&Sp->status, err);
  store_unit(A, U, u, set == kIntPre);
}

// Per-system totals in a fixed reduction order, out[kEnergyOut*s + c]: the five
// potential planes, the kinetic energy, then the virial tensor
// W_ab = Σ_i x_a F_b (row-major, kcal/mol) from the current forces.
__global__ void __launch_bounds__(256) k_energy_reduce(Arena A, double* out) {
  const int s = blockIdx.x;
  const SysDev S = A.sys[s];
  __shared__ double red[kEnergyOut][256];
  double acc[kEnergyOut];
  for (int c = 0; c < kEnergyOut; ++c) acc[c] = 0.0;
  if (S.active) {
    for (int i = threadIdx.x; i < S.n_atoms; i += blockDim.x) {
      const int a = S.atom_begin + i;
      for (int c = 0; c < 5; ++c) acc[c] += A.pe[(int64_t)c * A.atom_cap + a];
      double x[3], v[3], f[3], m;
      if (A.fp64) {
        const double4_32a p = A.pos64[a], w = A.vel64[a];
        x[0] = p.x; x[1] = p.y; x[2] = p.z;
        v[0] = w.x; v[1] = w.y; v[2] = w.z;
        m = w.w;
        for (int d = 0; d < 3; ++d) f[d] = A.f64[(int64_t)d * A.atom_cap + a];
      } else {
        const float4 p = A.pos[a], w = A.vel[a];
        x[0] = p.x; x[1] = p.y; x[2] = p.z;
        v[0] = w.x; v[1] = w.y; v[2] = w.z;
        m = w.w;
        for (int d = 0; d < 3; ++d) f[d] = (double)A.f[(int64_t)d * A.atom_cap + a] * kFixedInvD;
      }
      const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      acc[5] += 0.5 * m * v2 / (double)kKcalToAmuA2Ps2;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) acc[6 + 3 * r + c] += x[r] * f[c];
    }
  }
  for (int c = 0; c < kEnergyOut; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < kEnergyOut; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kEnergyOut) out[kEnergyOut * s + threadIdx.x] = red[threadIdx.x][0];
}

void launch_integrate(const Arena& A, int64_t n_units_span, int mode, cudaStream_t st, int check64_pass) {
  if (n_units_span <= 0) return;
  const unsigned blocks = (unsigned)((n_units_span + 127) / 128);
  if (A.fp64)
    k_integrate<double, false><<<blocks, 128, 0, st>>>(A, n_units_span, mode);
  else if (check64_pass)
    k_integrate<float, true><<<blocks, 128, 0, st>>>(A, n_units_span, mode);
  else
    k_integrate<float, false><<<blocks, 128, 0, st>>>(A, n_units_span, mode);
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
