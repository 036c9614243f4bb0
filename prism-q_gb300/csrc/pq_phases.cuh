// Integrator phase bodies shared by the fused integrate kernel and the
// per-system control kernel.  One call handles one constraint unit (an H
// cluster or a lone atom) entirely in registers, so every OU / kick / RATTLE /
// drift / SHAKE / clamp phase of the reference's per-phase launches becomes a
// straight-line sequence per unit.
//
// Arithmetic follows the reference phase bodies operation for operation
// (nhs_amber_fused.cu):
//   OU          langevin_thermostat                     :1713-1744, phases 10/15 :3656-3666
//   kick        apply_force_half_kick_with_...work      :1750-1787 (+ prism_asc_used_force)
//               apply_exact_force_half_kick (γ == 0)    :1792-1802
//   RATTLE      rattle_cluster_velocities               :2176-2268
//   drift       MD_PHASE_DRIFT_SAVE_XN                  :3780-3794
//   SHAKE       shake_cluster_positions                 :1890-2038
//   clamp       nhs_velocity_safety_clamp               :11148-11185
// This header is compiled without FMA contraction (--fmad=false) so that the
// CPU oracle, built with -ffp-contract=off, reproduces it bit for bit.
#pragma once

#include "pq_common.cuh"
#include "pq_device.cuh"

namespace pq {

// Loops over the (at most four) atoms of a unit are fully unrolled so the
// unit's state stays in registers; the order of operations is unchanged.
#define PQ_UNROLL _Pragma("unroll")

struct UnitState {
  float x[4], y[4], z[4];
  float vx[4], vy[4], vz[4];
  float m[4];
  float fx[4], fy[4], fz[4];
  int n;  // atoms in the unit
};

__device__ __forceinline__ void ou_half(UnitState& u, const SysDev& S, int atom_local0,
                                        const int* atom_local, uint64_t step, uint32_t purpose) {
  if (S.gamma == 0.0f) return;
  const float c1 = S.c1;
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const float c2 = sqrtf((1.0f - c1 * c1) * kKcalToAmuA2Ps2 * kBoltzmann * S.temperature / u.m[k]);
    float z0, z1, z2;
    normal3(S.seed, S.stream, (uint32_t)atom_local[k], step, purpose, &z0, &z1, &z2);
    u.vx[k] = c1 * u.vx[k] + c2 * z0;
    u.vy[k] = c1 * u.vy[k] + c2 * z1;
    u.vz[k] = c1 * u.vz[k] + c2 * z2;
  }
  (void)atom_local0;
}

__device__ __forceinline__ void half_kick(UnitState& u, const SysDev& S) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const float kick = 0.5f * S.dt * kKcalToAmuA2Ps2 / u.m[k];
    if (S.gamma == 0.0f) {
      u.vx[k] += kick * u.fx[k];
      u.vy[k] += kick * u.fy[k];
      u.vz[k] += kick * u.fz[k];
    } else {
      const float a = u.fx[k] * 1.0f, b = u.fy[k] * 1.0f, c = u.fz[k] * 1.0f;
      const float mag = sqrtf(a * a + b * b + c * c);
      const float q = mag > kMaxKickForce ? kMaxKickForce / mag : 1.0f;
      u.vx[k] = u.vx[k] + kick * (a * q);
      u.vy[k] = u.vy[k] + kick * (b * q);
      u.vz[k] = u.vz[k] + kick * (c * q);
    }
  }
}

// Returns false on non-convergence or invalid geometry.
__device__ __forceinline__ bool rattle(UnitState& u, const Unit& U, int max_iter) {
  const int nh = U.nh;
  if (nh <= 0) return true;
  const float tol = 1.0e-5f;
  const float ic = U.inv_mc, ih = U.inv_mh;
  for (int it = 0; it < max_iter; ++it) {
    float maxe = 0.0f;
    PQ_UNROLL for (int h = 1; h <= 3; ++h) {
      if (h > nh) break;
      const float rx = u.x[h] - u.x[0], ry = u.y[h] - u.y[0], rz = u.z[h] - u.z[0];
      const float r2 = rx * rx + ry * ry + rz * rz;
      if (!isfinite(r2) || r2 < 1.0e-12f) return false;
      const float wx = u.vx[h] - u.vx[0], wy = u.vy[h] - u.vy[0], wz = u.vz[h] - u.vz[0];
      const float res = rx * wx + ry * wy + rz * wz;
      const float spd = sqrtf(wx * wx + wy * wy + wz * wz);
      const float scale = sqrtf(r2) * fmaxf(spd, 1.0f);
      const float rel = fabsf(res) / scale;
      if (!isfinite(rel)) return false;
      maxe = fmaxf(maxe, rel);
      if (rel <= tol) continue;
      const float lam = res / ((ic + ih) * r2);
      const float cx = lam * rx, cy = lam * ry, cz = lam * rz;
      u.vx[0] += ic * cx;
      u.vy[0] += ic * cy;
      u.vz[0] += ic * cz;
      u.vx[h] -= ih * cx;
      u.vy[h] -= ih * cy;
      u.vz[h] -= ih * cz;
    }
    if (maxe <= tol) return true;
  }
  return false;
}

__device__ __forceinline__ bool shake(UnitState& u, const Unit& U, const float* sx, const float* sy,
                                      const float* sz, float dt, int max_iter) {
  const int nh = U.nh;
  if (nh <= 0) return true;
  const float tol = 1.0e-4f;
  const float ic = U.inv_mc, ih = U.inv_mh;
  for (int it = 0; it < max_iter; ++it) {
    float maxe = 0.0f;
    PQ_UNROLL for (int h = 1; h <= 3; ++h) {
      if (h > nh) break;
      const float rx = u.x[h] - u.x[0], ry = u.y[h] - u.y[0], rz = u.z[h] - u.z[0];
      const float ox = sx[h] - sx[0], oy = sy[h] - sy[0], oz = sz[h] - sz[0];
      const float r2 = rx * rx + ry * ry + rz * rz;
      const float L = U.r0[h - 1];
      const float t2 = L * L;
      const float diff = r2 - t2;
      if (!isfinite(r2) || !isfinite(t2) || t2 <= 0.0f) return false;
      const float rel = fabsf(diff) / t2;
      maxe = fmaxf(maxe, rel);
      if (rel <= tol) continue;
      const float rdo = rx * ox + ry * oy + rz * oz;
      const float o2 = ox * ox + oy * oy + oz * oz;
      const float ds = sqrtf(r2 * o2);
      if (!isfinite(rdo) || !isfinite(ds) || ds <= 0.0f || fabsf(rdo) / ds <= 1.0e-6f ||
          !isfinite(dt) || dt <= 0.0f)
        return false;
      const float lam = diff / (2.0f * (ic + ih) * rdo);
      const float cx = lam * ox, cy = lam * oy, cz = lam * oz;
      u.x[0] += ic * cx;
      u.y[0] += ic * cy;
      u.z[0] += ic * cz;
      u.x[h] -= ih * cx;
      u.y[h] -= ih * cy;
      u.z[h] -= ih * cz;
      u.vx[0] += ic * cx / dt;
      u.vy[0] += ic * cy / dt;
      u.vz[0] += ic * cz / dt;
      u.vx[h] -= ih * cx / dt;
      u.vy[h] -= ih * cy / dt;
      u.vz[h] -= ih * cz / dt;
    }
    if (maxe <= tol) return true;
  }
  return false;
}

__device__ __forceinline__ void velocity_clamp(UnitState& u, const SysDev& S) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const float thermal = sqrtf(kKcalToAmuA2Ps2 * kBoltzmann * S.temperature / fmaxf(u.m[k], 1.0f));
    const float vmax = fmaxf(20.0f * thermal, 2.0f);
    const float mag = sqrtf(u.vx[k] * u.vx[k] + u.vy[k] * u.vy[k] + u.vz[k] * u.vz[k]);
    if (mag <= vmax) continue;
    const float s = vmax / mag;
    u.vx[k] = u.vx[k] * s;
    u.vy[k] = u.vy[k] * s;
    u.vz[k] = u.vz[k] * s;
  }
}

__device__ __forceinline__ void load_unit(const Arena& A, const Unit& U, UnitState& u, int* local,
                                          int atom_begin) {
  u.n = U.nh < 0 ? 0 : 1 + U.nh;
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const int a = U.a[k];
    const float4 p = A.pos[a];
    const float4 v = A.vel[a];
    u.x[k] = p.x;
    u.y[k] = p.y;
    u.z[k] = p.z;
    u.vx[k] = v.x;
    u.vy[k] = v.y;
    u.vz[k] = v.z;
    u.m[k] = v.w;
    u.fx[k] = fixed2f(A.f[a]);
    u.fy[k] = fixed2f(A.f[A.atom_cap + a]);
    u.fz[k] = fixed2f(A.f[2 * A.atom_cap + a]);
    local[k] = a - atom_begin;
  }
}

__device__ __forceinline__ void store_unit(const Arena& A, const Unit& U, const UnitState& u) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const int a = U.a[k];
    const float4 p = A.pos[a];
    A.pos[a] = make_float4(u.x[k], u.y[k], u.z[k], p.w);
    A.vel[a] = make_float4(u.vx[k], u.vy[k], u.vz[k], u.m[k]);
  }
}

// Post-force phases of step s: KICK_NP1 → RATTLE_BEFORE_OU_NP1 → OU_HALF_NP1,
// then the post-step velocity clamp and final RATTLE (fused_engine.rs:17498-17800).
__device__ __forceinline__ int phases_post(UnitState& u, const Unit& U, const SysDev& S,
                                           const int* local, uint64_t s) {
  half_kick(u, S);
  if (!rattle(u, U, S.max_iter)) return kStRattle;
  ou_half(u, S, 0, local, s, kPurposeOuNp1);
  velocity_clamp(u, S);
  if (!rattle(u, U, S.max_iter)) return kStRattle;
  return 0;
}

// Pre-force phases of step s: OU_HALF_N → RATTLE_AFTER_OU_N → KICK_N →
// RATTLE_PRE_DRIFT → DRIFT_SAVE_XN → SHAKE_POSITION.
__device__ __forceinline__ int phases_pre(UnitState& u, const Unit& U, const SysDev& S,
                                          const int* local, uint64_t s) {
  ou_half(u, S, 0, local, s, kPurposeOuN);
  if (!rattle(u, U, S.max_iter)) return kStRattle;
  half_kick(u, S);
  if (!rattle(u, U, S.max_iter)) return kStRattle;
  float sx[4], sy[4], sz[4];
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    sx[k] = u.x[k];
    sy[k] = u.y[k];
    sz[k] = u.z[k];
    u.x[k] += S.dt * u.vx[k];
    u.y[k] += S.dt * u.vy[k];
    u.z[k] += S.dt * u.vz[k];
  }
  if (!shake(u, U, sx, sy, sz, S.dt, S.max_iter)) return kStShake;
  return 0;
}

__device__ __forceinline__ bool unit_finite(const UnitState& u) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    if (!isfinite(u.x[k]) || !isfinite(u.y[k]) || !isfinite(u.z[k]) || !isfinite(u.vx[k]) ||
        !isfinite(u.vy[k]) || !isfinite(u.vz[k]))
      return false;
  }
  return true;
}

// Displacement since the last list build beyond half the skin sets the
// system's rebuild trigger.
__device__ __forceinline__ void check_displacement(const Arena& A, const Unit& U, const UnitState& u,
                                                   SysDev* S) {
  bool moved = false;
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const float4 r = A.xref[U.a[k]];
    const float dx = u.x[k] - r.x, dy = u.y[k] - r.y, dz = u.z[k] - r.z;
    if (dx * dx + dy * dy + dz * dz > S->half_skin2) moved = true;
  }
  if (moved) atomicOr(&S->displaced, 1);
}

}  // namespace pq
