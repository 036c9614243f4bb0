// Reference-kernel harness — TEST INFRASTRUCTURE (oracle side), never linked
// into the product.
//
// Compiles the reference's own CUDA source (crates/prism-gpu/src/kernels/
// nhs_amber_fused.cu, included below from where it lies in the reference
// tree) into a device-only cubin, and adds thin __global__ wrappers that call
// the reference's device functions one term / one cluster / one atom per
// thread on caller-supplied arrays:
//   compute_bond_force            nhs_amber_fused.cu:355
//   compute_angle_force           :389
//   compute_dihedral_force        :525
//   compute_nonbonded_force       :644 (ordinary pairs and exact exceptions)
//   apply_force_half_kick_with_intervention_work  :1750
//   apply_exact_force_half_kick   :1792
//   langevin_thermostat           :1713 (the OU half-step of phases
//                                 OU_HALF_N / OU_HALF_NP1, :3656-3666)
//   shake_cluster_positions       :1890
//   rattle_cluster_velocities     :2176
// and the reference's nhs_velocity_safety_clamp kernel (:11148) is launched
// as it is.  The tests feed these the same inputs as the CPU oracle and pin
// the oracle to the reference's own arithmetic.  Inputs are validated on the
// host first (in-range indices, converging constraint clusters), so no
// reference failure path is reached.  Build: oracle/build_ref.py.
#include <cstdio>

#include "nhs_amber_fused.cu"

namespace {
__device__ __forceinline__ int tid1() { return blockIdx.x * blockDim.x + threadIdx.x; }
}  // namespace

// Bond term t: atoms ij[2t], ij[2t+1]; (r0, k) = p[2t], p[2t+1].
// out[2t+m] = force on member m; pe[2t+m] = its energy share.
extern "C" __global__ void refh_bonds(int n, const int* ij, const float* p, const float3* pos, float3* out,
                                      double* pe) {
  const int t = tid1();
  if (t >= n) return;
  float3 fi = make_float3(0.f, 0.f, 0.f), fj = fi;
  compute_bond_force(pos[ij[2 * t]], pos[ij[2 * t + 1]], p[2 * t], p[2 * t + 1], fi, fj, pe + 2 * t, 0, 1);
  out[2 * t] = fi;
  out[2 * t + 1] = fj;
}

// Angle term t: atoms ijk[3t..3t+2]; (theta0, k) = p[2t], p[2t+1].
extern "C" __global__ void refh_angles(int n, const int* ijk, const float* p, const float3* pos, float3* out,
                                       double* pe) {
  const int t = tid1();
  if (t >= n) return;
  float3 f0 = make_float3(0.f, 0.f, 0.f), f1 = f0, f2 = f0;
  compute_angle_force(pos[ijk[3 * t]], pos[ijk[3 * t + 1]], pos[ijk[3 * t + 2]], p[2 * t], p[2 * t + 1], f0, f1,
                      f2, pe + 3 * t, 0, 1, 2);
  out[3 * t] = f0;
  out[3 * t + 1] = f1;
  out[3 * t + 2] = f2;
}

// Torsion term t: atoms ijkl[4t..4t+3], periodicity per[t]; (phase, k) = p[2t], p[2t+1].
extern "C" __global__ void refh_dihedrals(int n, const int* ijkl, const int* per, const float* p,
                                          const float3* pos, float3* out, double* pe) {
  const int t = tid1();
  if (t >= n) return;
  float3 f0 = make_float3(0.f, 0.f, 0.f), f1 = f0, f2 = f0, f3 = f0;
  compute_dihedral_force(pos[ijkl[4 * t]], pos[ijkl[4 * t + 1]], pos[ijkl[4 * t + 2]], pos[ijkl[4 * t + 3]],
                         per[t], p[2 * t], p[2 * t + 1], f0, f1, f2, f3, pe + 4 * t, 0, 1, 2, 3);
  out[4 * t] = f0;
  out[4 * t + 1] = f1;
  out[4 * t + 2] = f2;
  out[4 * t + 3] = f3;
}

// Pair t: atoms ij[2t], ij[2t+1].  exact[t] = 1 for an exact 1-4 exception
// with (qq, sigma, epsilon) = ex[3t..3t+2]; otherwise an ordinary pair with
// per-atom charges and LJ parameters, subject to the function's own cutoff.
extern "C" __global__ void refh_pairs(int n, const int* ij, const int* exact, const float* ex, const float* q,
                                      const float* sigma, const float* epsilon, float cutoff_sq,
                                      const float3* pos, float3* out, double* pe) {
  const int t = tid1();
  if (t >= n) return;
  const int i = ij[2 * t], j = ij[2 * t + 1];
  const bool x14 = exact[t] != 0;
  float3 fi = make_float3(0.f, 0.f, 0.f), fj = fi;
  compute_nonbonded_force(pos[i], pos[j], q[i], q[j], sigma[i], epsilon[i], sigma[j], epsilon[j], fi, fj,
                          cutoff_sq, pe + 2 * t, 0, 1, x14, x14, x14 ? ex[3 * t] : 0.f,
                          x14 ? ex[3 * t + 1] : 0.f, x14 ? ex[3 * t + 2] : 0.f, false);
  out[2 * t] = fi;
  out[2 * t + 1] = fj;
}

// Half-kick of atom a with force f[a]: exact != 0 selects the gamma-zero
// Hamiltonian kick, otherwise the production kick with the 1000 kcal/mol/Å
// clamp at force scale 1.
extern "C" __global__ void refh_kick(int n, float3* vel, const float3* f, const float* mass, float dt, int exact) {
  const int a = tid1();
  if (a >= n) return;
  float3 v = vel[a];
  if (exact)
    apply_exact_force_half_kick(v, f[a], mass[a], dt);
  else
    apply_force_half_kick_with_intervention_work(v, f[a], 1.0f, mass[a], dt, nullptr);
  vel[a] = v;
}

// Cluster c: ci[5c..5c+4] = central, h0, h1, h2, n_h; cf[5c..5c+4] = bond
// lengths 0..2, inverse central mass, inverse hydrogen mass.
__device__ __forceinline__ HCluster refh_cluster(const int* ci, const float* cf, int c) {
  HCluster h;
  h.central_atom = ci[5 * c];
  for (int k = 0; k < 3; ++k) {
    h.hydrogen_atoms[k] = ci[5 * c + 1 + k];
    h.bond_lengths[k] = cf[5 * c + k];
  }
  h.n_hydrogens = ci[5 * c + 4];
  h.inv_mass_central = cf[5 * c + 3];
  h.inv_mass_h = cf[5 * c + 4];
  return h;
}

extern "C" __global__ void refh_rattle(int n, const int* ci, const float* cf, const float3* pos, float3* vel,
                                       int max_iter, int* ok) {
  const int c = tid1();
  if (c >= n) return;
  ok[c] = rattle_cluster_velocities<false>(pos, vel, refh_cluster(ci, cf, c), nullptr, max_iter) ? 1 : 0;
}

extern "C" __global__ void refh_shake(int n, const int* ci, const float* cf, float3* pos, const float3* pos0,
                                      float3* vel, float dt, int max_iter, int step, int* ok) {
  const int c = tid1();
  if (c >= n) return;
  ok[c] = shake_cluster_positions<false>(pos, pos0, vel, refh_cluster(ci, cf, c), dt, nullptr, max_iter, step)
              ? 1 : 0;
}

// The clamp kernel reads its temperature from a ProtocolState.
extern "C" __global__ void refh_protocol_size(int* out) { *out = (int)sizeof(ProtocolState); }

extern "C" __global__ void refh_protocol_init(ProtocolState* p, float temperature) {
  unsigned char* b = reinterpret_cast<unsigned char*>(p);
  for (int k = 0; k < (int)sizeof(ProtocolState); ++k) b[k] = 0;
  p->current_temperature = temperature;
}

// OU half-step of atom a by the reference's own thermostat, as the OU phases
// call it (langevin_thermostat with 0.5 dt, nhs_amber_fused.cu:3656-3666),
// from a cuRAND state initialised as init_rng_states does
// (curand_init(seed, a, 0), :11308).  The three normals the thermostat
// draws are recorded from a copy of that state, and c1 is evaluated as the
// thermostat evaluates it, so a restatement given the same normals and c1
// can be compared bit for bit.
extern "C" __global__ void refh_ou(int n, float3* vel, const float* mass, float temperature, float gamma, float dt,
                                   unsigned long long seed, float* normals, float* c1_out) {
  const int a = tid1();
  if (a >= n) return;
  curandState st;
  curand_init(seed, a, 0, &st);
  curandState cp = st;
  normals[3 * a] = curand_normal(&cp);
  normals[3 * a + 1] = curand_normal(&cp);
  normals[3 * a + 2] = curand_normal(&cp);
  const float dt_half = 0.5f * dt;
  float3 v = vel[a];
  langevin_thermostat(v, mass[a], temperature, gamma, dt_half, &st, nullptr);
  vel[a] = v;
  if (a == 0) c1_out[0] = expf(-gamma * dt_half);
}
