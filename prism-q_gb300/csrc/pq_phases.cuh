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
//
// Every body is a template over the real type R: R = float is the production
// (and reference) arithmetic; R = double is the FP64-everywhere run of the
// precision study, the same sequence of operations in double.  With kCheck64
// set, the FP32 path evaluates the constraint residuals and Lagrange
// multipliers in FP64 (the corrections are still applied in FP32).
#pragma once

#include <type_traits>

#include "pq_common.cuh"
#include "pq_device.cuh"

namespace pq {

// Loops over the (at most four) atoms of a unit are fully unrolled so the
// unit's state stays in registers; the order of operations is unchanged.
#define PQ_UNROLL _Pragma("unroll")

__device__ __forceinline__ float sqrt_r(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__device__ __forceinline__ float abs_r(float x) { return fabsf(x); }
__device__ __forceinline__ double abs_r(double x) { return fabs(x); }
__device__ __forceinline__ float max_r(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double max_r(double a, double b) { return fmax(a, b); }

// Constants in each precision: the FP32 path uses the reference's float
// literals; the FP64 path uses the same quantities in double.
template <class R>
struct PhaseConst;
template <>
struct PhaseConst<float> {
  static __device__ __forceinline__ float kcal() { return kKcalToAmuA2Ps2; }
  static __device__ __forceinline__ float kb() { return kBoltzmann; }
  static __device__ __forceinline__ float c1(const SysDev& S) { return S.c1; }
};
template <>
struct PhaseConst<double> {
  static __device__ __forceinline__ double kcal() { return 418.4; }
  static __device__ __forceinline__ double kb() { return 0.001987204; }
  static __device__ __forceinline__ double c1(const SysDev& S) { return S.c1d; }
};

template <class R>
struct UnitStateT {
  R x[4], y[4], z[4];
  R vx[4], vy[4], vz[4];
  R m[4];
  R fx[4], fy[4], fz[4];
  int n;  // atoms in the unit
};
using UnitState = UnitStateT<float>;

// OU half step.  With kDrawn the normals come from `znoise` (indexed by global
// atom, drawn ahead by k_noise with the same normal3); otherwise they are
// drawn here.
template <class R, bool kDrawn>
__device__ __forceinline__ void ou_half(UnitStateT<R>& u, const Unit& U, const SysDev& S, const int* atom_local,
                                        uint64_t step, uint32_t purpose, const float4* znoise) {
  if (S.gamma == 0.0f) return;
  const R c1 = PhaseConst<R>::c1(S);
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const R c2 = sqrt_r((R(1.0f) - c1 * c1) * PhaseConst<R>::kcal() * PhaseConst<R>::kb() * R(S.temperature) / u.m[k]);
    float z0, z1, z2;
    if constexpr (kDrawn) {
      const float4 z = znoise[U.a[k]];
      z0 = z.x;
      z1 = z.y;
      z2 = z.z;
    } else {
      normal3(S.seed, S.stream, (uint32_t)atom_local[k], step, purpose, &z0, &z1, &z2);
    }
    u.vx[k] = c1 * u.vx[k] + c2 * R(z0);
    u.vy[k] = c1 * u.vy[k] + c2 * R(z1);
    u.vz[k] = c1 * u.vz[k] + c2 * R(z2);
  }
}

template <class R>
__device__ __forceinline__ void half_kick(UnitStateT<R>& u, const SysDev& S) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const R kick = R(0.5f) * R(S.dt) * PhaseConst<R>::kcal() / u.m[k];
    if (S.gamma == 0.0f) {
      u.vx[k] += kick * u.fx[k];
      u.vy[k] += kick * u.fy[k];
      u.vz[k] += kick * u.fz[k];
    } else {
      const R a = u.fx[k] * R(1.0f), b = u.fy[k] * R(1.0f), c = u.fz[k] * R(1.0f);
      const R mag = sqrt_r(a * a + b * b + c * c);
      const R q = mag > R(kMaxKickForce) ? R(kMaxKickForce) / mag : R(1.0f);
      u.vx[k] = u.vx[k] + kick * (a * q);
      u.vy[k] = u.vy[k] + kick * (b * q);
      u.vz[k] = u.vz[k] + kick * (c * q);
    }
  }
}

// One RATTLE velocity correction for hydrogen h.  Returns the relative residual
// before the correction (negative on invalid geometry).  The residual and the
// multiplier are evaluated in type C (C = R, or double for kCheck64).
template <class R, class C>
__device__ __forceinline__ C rattle_one(UnitStateT<R>& u, int h, R ic, R ih, C tol) {
  const C rx = C(u.x[h]) - C(u.x[0]), ry = C(u.y[h]) - C(u.y[0]), rz = C(u.z[h]) - C(u.z[0]);
  const C r2 = rx * rx + ry * ry + rz * rz;
  if (!isfinite(r2) || r2 < C(1.0e-12f)) return C(-1.0f);
  const C wx = C(u.vx[h]) - C(u.vx[0]), wy = C(u.vy[h]) - C(u.vy[0]), wz = C(u.vz[h]) - C(u.vz[0]);
  const C res = rx * wx + ry * wy + rz * wz;
  const C spd = sqrt_r(wx * wx + wy * wy + wz * wz);
  const C scale = sqrt_r(r2) * max_r(spd, C(1.0f));
  const C rel = abs_r(res) / scale;
  if (!isfinite(rel)) return C(-1.0f);
  if (rel <= tol) return rel;
  const C lam = res / ((C(ic) + C(ih)) * r2);
  const R cx = R(lam * rx), cy = R(lam * ry), cz = R(lam * rz);
  u.vx[0] += ic * cx;
  u.vy[0] += ic * cy;
  u.vz[0] += ic * cz;
  u.vx[h] -= ih * cx;
  u.vy[h] -= ih * cy;
  u.vz[h] -= ih * cz;
  return rel;
}

// Returns false on non-convergence or invalid geometry.
template <class R, bool kCheck64>
__device__ __forceinline__ bool rattle(UnitStateT<R>& u, const Unit& U, const SysDev& S) {
  using C = typename std::conditional<kCheck64, double, R>::type;
  const int nh = U.nh;
  if (nh <= 0) return true;
  const C tol = C(S.rattle_tol);
  const R ic = R(U.inv_mc), ih = R(U.inv_mh);
  for (int it = 0; it < S.max_iter; ++it) {
    C maxe = C(0.0f);
    PQ_UNROLL for (int h = 1; h <= 3; ++h) {
      if (h > nh) break;
      const C rel = rattle_one<R, C>(u, h, ic, ih, tol);
      if (rel < C(0.0f)) return false;
      maxe = max_r(maxe, rel);
    }
    if (maxe <= tol) return true;
  }
  return false;
}

// One SHAKE position correction for hydrogen h along the step-start bond.
// Returns the relative residual before the correction (negative on invalid
// geometry).
template <class R, class C>
__device__ __forceinline__ C shake_one(UnitStateT<R>& u, const Unit& U, int h, const R* sx, const R* sy,
                                       const R* sz, R dt, R ic, R ih, C tol) {
  const C rx = C(u.x[h]) - C(u.x[0]), ry = C(u.y[h]) - C(u.y[0]), rz = C(u.z[h]) - C(u.z[0]);
  const C ox = C(sx[h]) - C(sx[0]), oy = C(sy[h]) - C(sy[0]), oz = C(sz[h]) - C(sz[0]);
  const C r2 = rx * rx + ry * ry + rz * rz;
  const C L = C(U.r0[h - 1]);
  const C t2 = L * L;
  const C diff = r2 - t2;
  if (!isfinite(r2) || !isfinite(t2) || t2 <= C(0.0f)) return C(-1.0f);
  const C rel = abs_r(diff) / t2;
  if (rel <= tol) return rel;
  const C rdo = rx * ox + ry * oy + rz * oz;
  const C o2 = ox * ox + oy * oy + oz * oz;
  const C ds = sqrt_r(r2 * o2);
  if (!isfinite(rdo) || !isfinite(ds) || ds <= C(0.0f) || abs_r(rdo) / ds <= C(1.0e-6f) || !isfinite(dt) ||
      dt <= R(0.0f))
    return C(-1.0f);
  const C lam = diff / (C(2.0f) * (C(ic) + C(ih)) * rdo);
  const R cx = R(lam * ox), cy = R(lam * oy), cz = R(lam * oz);
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
  return rel;
}

template <class R, bool kCheck64>
__device__ __forceinline__ bool shake(UnitStateT<R>& u, const Unit& U, const R* sx, const R* sy, const R* sz,
                                      const SysDev& S) {
  using C = typename std::conditional<kCheck64, double, R>::type;
  const int nh = U.nh;
  if (nh <= 0) return true;
  const C tol = C(S.shake_tol);
  const R ic = R(U.inv_mc), ih = R(U.inv_mh), dt = R(S.dt);
  for (int it = 0; it < S.max_iter; ++it) {
    C maxe = C(0.0f);
    PQ_UNROLL for (int h = 1; h <= 3; ++h) {
      if (h > nh) break;
      const C rel = shake_one<R, C>(u, U, h, sx, sy, sz, dt, ic, ih, tol);
      if (rel < C(0.0f)) return false;
      maxe = max_r(maxe, rel);
    }
    if (maxe <= tol) return true;
  }
  return false;
}

template <class R>
__device__ __forceinline__ void velocity_clamp(UnitStateT<R>& u, const SysDev& S) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const R thermal = sqrt_r(PhaseConst<R>::kcal() * PhaseConst<R>::kb() * R(S.temperature) / max_r(u.m[k], R(1.0f)));
    const R vmax = max_r(R(20.0f) * thermal, R(2.0f));
    const R mag = sqrt_r(u.vx[k] * u.vx[k] + u.vy[k] * u.vy[k] + u.vz[k] * u.vz[k]);
    if (mag <= vmax) continue;
    const R s = vmax / mag;
    u.vx[k] = u.vx[k] * s;
    u.vy[k] = u.vy[k] * s;
    u.vz[k] = u.vz[k] * s;
  }
}

__device__ __forceinline__ void load_unit(const Arena& A, const Unit& U, UnitStateT<float>& u, int* local,
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

__device__ __forceinline__ void load_unit(const Arena& A, const Unit& U, UnitStateT<double>& u, int* local,
                                          int atom_begin) {
  u.n = U.nh < 0 ? 0 : 1 + U.nh;
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const int a = U.a[k];
    const double4_32a p = A.pos64[a];
    const double4_32a v = A.vel64[a];
    u.x[k] = p.x;
    u.y[k] = p.y;
    u.z[k] = p.z;
    u.vx[k] = v.x;
    u.vy[k] = v.y;
    u.vz[k] = v.z;
    u.m[k] = v.w;
    u.fx[k] = A.f64[a];
    u.fy[k] = A.f64[A.atom_cap + a];
    u.fz[k] = A.f64[2 * A.atom_cap + a];
    local[k] = a - atom_begin;
  }
}

// `moved`: the positions changed and are written back.
__device__ __forceinline__ void store_unit(const Arena& A, const Unit& U, const UnitStateT<float>& u, bool moved) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const int a = U.a[k];
    if (moved) A.pos[a] = make_float4(u.x[k], u.y[k], u.z[k], A.pos[a].w);
    A.vel[a] = make_float4(u.vx[k], u.vy[k], u.vz[k], u.m[k]);
  }
}

// FP64 state plus its FP32 rounding, which the cell and row kernels read.
__device__ __forceinline__ void store_unit(const Arena& A, const Unit& U, const UnitStateT<double>& u, bool moved) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const int a = U.a[k];
    if (moved) {
      A.pos64[a] = make_double4_32a(u.x[k], u.y[k], u.z[k], A.pos64[a].w);
      A.pos[a] = make_float4((float)u.x[k], (float)u.y[k], (float)u.z[k], A.pos[a].w);
    }
    A.vel64[a] = make_double4_32a(u.vx[k], u.vy[k], u.vz[k], u.m[k]);
    A.vel[a] = make_float4((float)u.vx[k], (float)u.vy[k], (float)u.vz[k], (float)u.m[k]);
  }
}

// Post-force phases of step s: KICK_NP1 → RATTLE_BEFORE_OU_NP1 → OU_HALF_NP1,
// then the post-step velocity clamp and final RATTLE (fused_engine.rs:17498-17800).
template <class R, bool kCheck64, bool kDrawn = false>
__device__ __forceinline__ int phases_post(UnitStateT<R>& u, const Unit& U, const SysDev& S, const int* local,
                                           uint64_t s, const float4* znoise = nullptr) {
  half_kick(u, S);
  if (!rattle<R, kCheck64>(u, U, S)) return kStRattle;
  ou_half<R, kDrawn>(u, U, S, local, s, kPurposeOuNp1, znoise);
  velocity_clamp(u, S);
  if (!rattle<R, kCheck64>(u, U, S)) return kStRattle;
  return 0;
}

// Pre-force phases of step s: OU_HALF_N → RATTLE_AFTER_OU_N → KICK_N →
// RATTLE_PRE_DRIFT → DRIFT_SAVE_XN → SHAKE_POSITION.
template <class R, bool kCheck64, bool kDrawn = false>
__device__ __forceinline__ int phases_pre(UnitStateT<R>& u, const Unit& U, const SysDev& S, const int* local,
                                          uint64_t s, const float4* znoise = nullptr) {
  ou_half<R, kDrawn>(u, U, S, local, s, kPurposeOuN, znoise);
  if (!rattle<R, kCheck64>(u, U, S)) return kStRattle;
  half_kick(u, S);
  if (!rattle<R, kCheck64>(u, U, S)) return kStRattle;
  R sx[4], sy[4], sz[4];
  const R dt = R(S.dt);
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    sx[k] = u.x[k];
    sy[k] = u.y[k];
    sz[k] = u.z[k];
    u.x[k] += dt * u.vx[k];
    u.y[k] += dt * u.vy[k];
    u.z[k] += dt * u.vz[k];
  }
  if (!shake<R, kCheck64>(u, U, sx, sy, sz, S)) return kStShake;
  return 0;
}

template <class R>
__device__ __forceinline__ bool unit_finite(const UnitStateT<R>& u) {
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    if (!isfinite(u.x[k]) || !isfinite(u.y[k]) || !isfinite(u.z[k]) || !isfinite(u.vx[k]) ||
        !isfinite(u.vy[k]) || !isfinite(u.vz[k]))
      return false;
  }
  return true;
}

// Displacement since the last list build beyond half the skin sets the
// system's rebuild trigger (measured on the FP32 positions the lists use).
template <class R>
__device__ __forceinline__ void check_displacement(const Arena& A, const Unit& U, const UnitStateT<R>& u,
                                                   SysDev* S) {
  bool moved = false;
  PQ_UNROLL for (int k = 0; k < 4; ++k) {
    if (k >= u.n) break;
    const float4 r = A.xref[U.a[k]];
    const float dx = (float)u.x[k] - r.x, dy = (float)u.y[k] - r.y, dz = (float)u.z[k] - r.z;
    if (dx * dx + dy * dy + dz * dz > S->half_skin2) moved = true;
  }
  if (moved) atomicOr(&S->displaced, 1);
}

}  // namespace pq
