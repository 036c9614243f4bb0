// Shared host/device definitions for the Prism-Q MD step on GB300.
//
// Everything in this header compiles both as CUDA device code and as plain
// host C++ (the host copy backs the noise/debug entry points and the topology
// lowering).  Functions whose results must be bit-identical on the GPU and on
// the host use only IEEE-exact operations (+ - * / sqrt, explicit fmaf) and
// integer arithmetic; the translation units that include them are compiled
// without floating-point contraction (host: -ffp-contract=off, device:
// --fmad=false for the integrator) so that `a*b+c` is never silently fused.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define PQ_HD __host__ __device__ __forceinline__
#else
#define PQ_HD inline
#endif

namespace pq {

// ---------------------------------------------------------------------------
// Units and physical constants of the reference engine.
// Units: Å, ps, amu, kcal/mol, e.  (nhs_amber_fused.cu:64-68)
// ---------------------------------------------------------------------------
constexpr float kCoulomb = 332.0636f;       // kcal·Å/(mol·e²)
constexpr float kKcalToAmuA2Ps2 = 418.4f;   // kcal/mol -> amu·Å²/ps²
constexpr float kBoltzmann = 0.001987204f;  // kcal/(mol·K)
constexpr float kMaxKickForce = 1000.0f;    // |λF| clamp of the half-kick
constexpr float kNonbondedCutoff = 10.0f;   // Å, potential cutoff
constexpr float kMinPairR2 = 0.01f;         // Å², ordinary pairs closer than this are skipped

// Fixed-point force representation: int64 at 2^-32 kcal/mol/Å per unit.
constexpr float kFixedScale = 4294967296.0f;          // 2^32
constexpr float kFixedInv = 2.3283064365386963e-10f;  // 2^-32
constexpr double kFixedInvD = 2.3283064365386963e-10;

// Noise purposes (the 8-bit purpose field of the Philox counter).
constexpr uint32_t kPurposeOuN = 1;    // OU half-step before the first kick
constexpr uint32_t kPurposeOuNp1 = 2;  // OU half-step after the second kick

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
// Keyed by (seed, stream); counter (atom, step_lo, step_hi16|purpose8|epoch8, 0),
// the same injective packing as scripts/physics_refs/rng_streams.py:80-84.
// ---------------------------------------------------------------------------
struct U32x4 {
  uint32_t v[4];
};

PQ_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

PQ_HD U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += W0;
      k1 += W1;
    }
    const uint32_t lo0 = M0 * c.v[0], hi0 = mulhi32(M0, c.v[0]);
    const uint32_t lo1 = M1 * c.v[2], hi1 = mulhi32(M1, c.v[2]);
    U32x4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
  }
  return c;
}

PQ_HD U32x4 keyed_draw(uint32_t seed, uint32_t stream, uint32_t epoch, uint32_t atom,
                       uint64_t step, uint32_t purpose) {
  U32x4 c;
  c.v[0] = atom;
  c.v[1] = (uint32_t)(step & 0xffffffffu);
  c.v[2] = ((uint32_t)((step >> 32) & 0xffffu) << 16) | ((purpose & 0xffu) << 8) | (epoch & 0xffu);
  c.v[3] = 0u;
  return philox4x32_10(c, seed, stream);
}

// ---------------------------------------------------------------------------
// Bit-reproducible normal deviates (Box–Muller with project-written ln/sin/cos).
//
// The transcendental pieces are written from their series definitions so that
// host and device produce identical bits:
//   ln m  = 2·atanh(s) = 2(s + s³/3 + s⁵/5 + …),  s = (m-1)/(m+1), m∈[√½,√2)
//   sin θ = θ - θ³/3! + …,  cos θ = 1 - θ²/2! + …,  θ∈[0, π/4]
// Every step is an IEEE-exact operation or an explicit fmaf.
// ---------------------------------------------------------------------------
PQ_HD float bits_to_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  union {
    uint32_t u;
    float f;
  } x;
  x.u = b;
  return x.f;
#endif
}
PQ_HD uint32_t float_to_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  union {
    uint32_t u;
    float f;
  } x;
  x.f = f;
  return x.u;
#endif
}
PQ_HD float exact_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// ln(u) for u in (0, 1], |rel err| ~ 1e-7.
PQ_HD float series_log(float u) {
  const uint32_t b = float_to_bits(u);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = bits_to_float((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = exact_fma(s2, 0.11111111f, 0.14285715f);  // 1/9, 1/7
  p = exact_fma(s2, p, 0.2f);                          // 1/5
  p = exact_fma(s2, p, 0.33333334f);                   // 1/3
  p = exact_fma(s2, p, 1.0f);
  const float two_s = s + s;
  return exact_fma((float)e, 0.69314718f, two_s * p);
}

// sin and cos of θ ∈ [0, π/4].
PQ_HD void series_sincos_octant(float t, float* sn, float* cs) {
  const float t2 = t * t;
  float ps = exact_fma(t2, 2.7557319e-06f, -1.9841270e-04f);  // 1/9!, -1/7!
  ps = exact_fma(t2, ps, 8.3333333e-03f);                     // 1/5!
  ps = exact_fma(t2, ps, -1.6666667e-01f);                    // -1/3!
  ps = exact_fma(t2, ps, 1.0f);
  float pc = exact_fma(t2, -2.7557319e-07f, 2.4801587e-05f);  // -1/10!, 1/8!
  pc = exact_fma(t2, pc, -1.3888889e-03f);                    // -1/6!
  pc = exact_fma(t2, pc, 4.1666667e-02f);                     // 1/4!
  pc = exact_fma(t2, pc, -0.5f);                              // -1/2!
  pc = exact_fma(t2, pc, 1.0f);
  *sn = t * ps;
  *cs = pc;
}

// cos(2πu), sin(2πu) for u = k·2^-24 in [0, 1).
PQ_HD void turn_sincos(float u, float* c, float* s) {
  const float t = u * 4.0f;              // exact
  const int q = (int)t;                  // quadrant 0..3
  float f = t - (float)q;                // [0,1), exact
  const bool flip = f > 0.5f;
  if (flip) f = 1.0f - f;                // exact
  float sn, cs;
  series_sincos_octant(f * 1.57079633f, &sn, &cs);
  if (flip) {
    const float tmp = sn;
    sn = cs;
    cs = tmp;
  }
  // (cos, sin) of (q·π/2 + θ)
  switch (q & 3) {
    case 0: *c = cs;  *s = sn;  break;
    case 1: *c = -sn; *s = cs;  break;
    case 2: *c = -cs; *s = -sn; break;
    default: *c = sn; *s = -cs; break;
  }
}

// Three standard normal deviates for (atom, step, purpose) of a system stream.
PQ_HD void normal3(uint32_t seed, uint32_t stream, uint32_t atom, uint64_t step, uint32_t purpose,
                   float* z0, float* z1, float* z2) {
  const U32x4 r = keyed_draw(seed, stream, 0u, atom, step, purpose);
  const float inv24 = 5.9604645e-08f;  // 2^-24
  const float u1 = (float)((r.v[0] >> 8) + 1u) * inv24;  // (0, 1]
  const float u2 = (float)(r.v[1] >> 8) * inv24;         // [0, 1)
  const float u3 = (float)((r.v[2] >> 8) + 1u) * inv24;
  const float u4 = (float)(r.v[3] >> 8) * inv24;
  const float ra = sqrtf(-2.0f * series_log(u1));
  const float rb = sqrtf(-2.0f * series_log(u3));
  float ca, sa, cb, sb;
  turn_sincos(u2, &ca, &sa);
  turn_sincos(u4, &cb, &sb);
  *z0 = ra * ca;
  *z1 = ra * sa;
  *z2 = rb * cb;
  (void)sb;
}

// ---------------------------------------------------------------------------
// Fixed-point helpers.  Device conversions saturate and map NaN to 0 (PTX
// cvt.rni.s64.f32); the host copy states the same rule explicitly.
// ---------------------------------------------------------------------------
PQ_HD long long f2fixed(float v) {
  const float s = v * kFixedScale;
#if defined(__CUDA_ARCH__)
  return __float2ll_rn(s);
#else
  if (s != s) return 0;
  if (s >= 9.2233720368547758e18f) return (long long)0x7fffffffffffffffLL;
  if (s <= -9.2233720368547758e18f) return (long long)(-0x7fffffffffffffffLL - 1);
  return llrintf(s);
#endif
}
PQ_HD float fixed2f(long long v) {
#if defined(__CUDA_ARCH__)
  return __ll2float_rn(v) * kFixedInv;
#else
  return (float)v * kFixedInv;
#endif
}

}  // namespace pq
