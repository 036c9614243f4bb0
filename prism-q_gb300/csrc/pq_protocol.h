// Per-step run protocol: temperature schedule, friction and timestep.
//
// Restates the reference's ProtocolState director (protocol_director.cu:54-143
// prism_protocol_baseline_v1, fields protocol_state.cuh:14-62, built by
// ProtocolState::from_cryo_uv, protocol_state.rs:602-700; the engine's
// compute_cryo_friction, fused_engine.rs:15366-15396):
//   temperature  5-phase schedule: cold hold -> linear ramp up -> warm hold ->
//                linear ramp down -> cold return (the warm temperature is kept
//                when the protocol has no cooling phases);
//   friction     exponential blend from the equilibration friction to the base
//                friction over the first equilibration steps, scaled by
//                sqrt(300 / max(T, 10)) below 300 K when cryo scaling is on;
//   timestep     adaptive mode 1: base dt in holds, base/2 in ramps; mode 2:
//                1.5 base in holds, base in ramps; mode 0: base dt.
// The director evaluates its own 1-based step counter: the first step after
// installation is director step current_step + 1 (protocol_director.cu:308-311).
//
// Every floating-point operation is an explicitly rounded IEEE operation
// (no contraction), and e^x is the project's binary64 series below, so the
// host and the device produce the same bits.  UV burst scheduling, steering
// hints and phase metrology of the reference struct are not part of the MD
// step and are not carried.
#pragma once

#include <stdint.h>

#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define PQ_HD __host__ __device__ __forceinline__
#else
#define PQ_HD inline
#endif

namespace pq {

PQ_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
PQ_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
PQ_HD float sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
PQ_HD float div_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
PQ_HD float sqrt_rn(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
PQ_HD double dmul_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
PQ_HD double dadd_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

// e^x in binary64: x = k ln2 + r with |r| <= ln2/2 (ln 2 split into a
// float-exact head and a binary64 tail, so k * head is exact), e^r by its
// Taylor series to degree 17 in Horner form (truncation below 1e-20
// relative), then scaled by 2^k built from its exponent bits.  Arguments
// below -708 return 0 (their float images are 0); the project uses this for
// arguments in [-1e4, 0].
PQ_HD double det_exp(double x) {
  if (!(x == x)) return x;
  if (x < -708.0) return 0.0;
  if (x > 709.0) return HUGE_VAL;
  const double ln2 = 0.69314718055994530941723212145818;
  const double head = (double)(float)ln2;
  const double tail = ln2 - head;
  const double kd = std::floor(dadd_rn(x / ln2, 0.5));
  const int k = (int)kd;
  const double r = dadd_rn(dadd_rn(x, -dmul_rn(kd, head)), -dmul_rn(kd, tail));
  // 1/n! for n = 17 .. 2, then 1, 1
  double p = 1.0 / 355687428096000.0;
  const double inv_fact[16] = {1.0 / 20922789888000.0, 1.0 / 1307674368000.0, 1.0 / 87178291200.0,
                               1.0 / 6227020800.0,     1.0 / 479001600.0,     1.0 / 39916800.0,
                               1.0 / 3628800.0,        1.0 / 362880.0,        1.0 / 40320.0,
                               1.0 / 5040.0,           1.0 / 720.0,           1.0 / 120.0,
                               1.0 / 24.0,             1.0 / 6.0,             1.0 / 2.0,
                               1.0};
  for (int q = 0; q < 16; ++q) p = dadd_rn(dmul_rn(p, r), inv_fact[q]);
  p = dadd_rn(dmul_rn(p, r), 1.0);
  const uint64_t bits = (uint64_t)(k + 1023) << 52;
#if defined(__CUDA_ARCH__)
  const double scale = __longlong_as_double((long long)bits);
#else
  double scale;
  std::memcpy(&scale, &bits, sizeof(scale));
#endif
  return dmul_rn(p, scale);
}

// Device form of a protocol.  Phase boundaries are director steps.
struct ProtocolDev {
  int on;
  int adaptive;   // 0 off, 1 bounded, 2 historical
  int cryo;
  int warm_tail;  // no cooling phases: the warm temperature persists
  int cold_hold_end, ramp_end, warm_hold_end, ramp_down_end;
  int equil_steps;
  float start_temp, end_temp, gamma_base, equil_gamma, base_dt;
  long long origin;  // director step = engine step - origin
};

struct StepParams {
  float temperature, gamma, dt, c1;
  double c1d;
};

// exp(-γ·dt/2): the OU coefficient for float and FP64 systems.
PQ_HD void ou_coefficients(StepParams* o) {
  const float arg = -mul_rn(o->gamma, mul_rn(0.5f, o->dt));
  o->c1 = (float)det_exp((double)arg);
  o->c1d = det_exp(dmul_rn(dmul_rn(-(double)o->gamma, 0.5), (double)o->dt));
}

// The director's values for one director step (prism_protocol_baseline_v1).
PQ_HD void protocol_eval(const ProtocolDev& P, long long director_step, StepParams* o) {
  const int s = director_step > 2147483647LL ? 2147483647 : (director_step < -2147483647LL ? -2147483647 : (int)director_step);
  float temp;
  int hold;
  if (s < P.cold_hold_end) {
    temp = P.start_temp;
    hold = 1;
  } else if (s < P.ramp_end) {
    const float progress = div_rn((float)(s - P.cold_hold_end), (float)(P.ramp_end - P.cold_hold_end));
    temp = add_rn(P.start_temp, mul_rn(progress, sub_rn(P.end_temp, P.start_temp)));
    hold = 0;
  } else if (s < P.warm_hold_end) {
    temp = P.end_temp;
    hold = 1;
  } else if (s < P.ramp_down_end) {
    const float progress = div_rn((float)(s - P.warm_hold_end), (float)(P.ramp_down_end - P.warm_hold_end));
    temp = sub_rn(P.end_temp, mul_rn(progress, sub_rn(P.end_temp, P.start_temp)));
    hold = 0;
  } else {
    temp = P.warm_tail ? P.end_temp : P.start_temp;
    hold = 1;
  }
  float base;
  if (s < P.equil_steps) {
    const float progress = div_rn((float)s, (float)P.equil_steps);
    const float decay = (float)det_exp((double)mul_rn(-3.0f, progress));
    base = add_rn(mul_rn(P.equil_gamma, decay), mul_rn(P.gamma_base, sub_rn(1.0f, decay)));
  } else {
    base = P.gamma_base;
  }
  float gamma = base;
  if (P.cryo && temp < 300.0f) {
    const float tc = temp > 10.0f ? temp : 10.0f;
    gamma = mul_rn(base, sqrt_rn(div_rn(300.0f, tc)));
  }
  float dt = P.base_dt;
  if (P.adaptive == 2)
    dt = hold ? mul_rn(P.base_dt, 1.5f) : P.base_dt;
  else if (P.adaptive == 1)
    dt = hold ? P.base_dt : mul_rn(P.base_dt, 0.5f);
  o->temperature = temp;
  o->gamma = gamma;
  o->dt = dt;
  ou_coefficients(o);
}

}  // namespace pq
