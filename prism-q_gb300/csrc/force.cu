// AMBER ff14SB force evaluation (FORCE_N / FORCE_NP1 phases).
//
// Reference: prism_amber_phase_body_v1, deterministic-gather branch
// (nhs_amber_fused.cu:2993-3484): one thread per atom gathers its bonded
// terms through incidence lists (every term recomputed by each member atom),
// its ordinary pairs from a full neighbour row (skip r^2 >= cutoff^2 or
// r^2 < 0.01, skip exception pairs), then its exact 1-4 exceptions (no cutoff,
// no shift), and writes its own force row.  Force laws: compute_bond_force
// :355, compute_angle_force :389, compute_dihedral_force :525 (OpenMM torsion
// gradient, asin branch for |cos φ| > 0.99), compute_nonbonded_force :644 and
// ordinary_cutoff_potential_offset_v1 :632.
//
// GB300 form: the same ownership (no force atomics), but
//   * positions+charges stream as float4 and LJ as float2 (σ/2, √ε);
//   * neighbour rows are interleaved by 8-atom group so that a lane reads its
//     next four row indices as one int4 and a warp's index loads are one
//     contiguous 512-byte block, and exception pairs are already excluded
//     from the rows (no per-neighbour 1-4 scan);
//   * partial sums are FP32 over at most 32 pairs and then accumulated in
//     int64 fixed point at 2^-32 kcal/mol/Å, so the force of an atom is a
//     deterministic function of its own row alone;
//   * energies are computed only by the energy variant (FP64 per-atom planes);
//   * the file is compiled without FMA contraction (the pair law's FMAs are
//     written out) and with subnormals flushed to zero, which changes no
//     IEEE-rounded result on normal values.
//
// The kernel is a template over the real type R.  R = float is the production
// path above.  R = double is the FP64-everywhere run of the precision study:
// the same decomposition with double positions, double pair and bonded math
// and double accumulation (lanes summed by the same fixed butterfly), writing
// the FP64 force planes.
#include <algorithm>

#include "pq_common.cuh"
#include "pq_device.cuh"

namespace pq {

template <class R>
struct Real4;
template <>
struct Real4<float> {
  using T = float4;
};
template <>
struct Real4<double> {
  using T = double4_32a;
};
template <class R>
using R4 = typename Real4<R>::T;

template <class R>
struct Real2;
template <>
struct Real2<float> {
  using T = float2;
};
template <>
struct Real2<double> {
  using T = double2;
};
template <class R>
using R2 = typename Real2<R>::T;

__device__ __forceinline__ const float4* positions(const Arena& A, float) { return A.pos; }
__device__ __forceinline__ const double4_32a* positions(const Arena& A, double) { return A.pos64; }
__device__ __forceinline__ const float2* lj_params(const Arena& A, float) { return A.lj; }
__device__ __forceinline__ const double2* lj_params(const Arena& A, double) { return A.lj64; }

// read-only gathers: float4 is one 16-byte load, double4 two 16-byte loads
__device__ __forceinline__ float4 ldg_r4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ double4_32a ldg_r4(const double4_32a* p) {
  const double2 lo = __ldg(reinterpret_cast<const double2*>(p));
  const double2 hi = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return make_double4_32a(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float sqrt_r(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__device__ __forceinline__ float acos_r(float x) { return acosf(x); }
__device__ __forceinline__ double acos_r(double x) { return acos(x); }
__device__ __forceinline__ float inv_sqrt_r(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt_r(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float min_r(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double min_r(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float max_r(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double max_r(double a, double b) { return fmax(a, b); }

// Force accumulator.  FP32: partial sums over at most 32 contributions, then
// int64 fixed point (exact, order-free).  FP64: plain double sums.
template <class R>
struct Acc;
template <>
struct Acc<float> {
  float x, y, z;
  long long X, Y, Z;
  __device__ __forceinline__ void flush() {
    X += f2fixed(x);
    Y += f2fixed(y);
    Z += f2fixed(z);
    x = y = z = 0.0f;
  }
};
template <>
struct Acc<double> {
  double x, y, z;
  __device__ __forceinline__ void flush() {}
};

// ---- pair law: force on i from j (d = xj - xi), LJ + Coulomb ----
// The file is compiled without FMA contraction, so every fused multiply-add
// is written out: the compiler cannot fuse differently in different launch
// shapes (register budgets), and every shape gives the same bits.
template <class R>
__device__ __forceinline__ R pair_scalar(R r2, R sig, R eps, R qq, R& inv_r, R& s6) {
  inv_r = inv_sqrt_r(r2);
  const R inv_r2 = inv_r * inv_r;
  const R s2 = sig * sig * inv_r2;
  s6 = s2 * s2 * s2;
  const R u = fma_r(R(2.0f) * s6, s6, -s6);            // 2 s6^2 - s6
  const R fc = R(kCoulomb) * qq * inv_r2 * inv_r;
  return fma_r(R(24.0f) * eps * inv_r2, u, fc);        // 24 eps/r^2 (2 s6^2 - s6) + qq k/r^3
}

// The same law for an ordinary pair with atom i's factors taken out of the
// pair: kqi = 332.0636·q_i and e24i = 24·√ε_i (LJ parameters hold √ε), so
// the pair costs three multiplications fewer:
// fs = (24 ε (2 s6² − s6) + k q_i q_j / r) / r², with s6 = (σ/r)^6.
template <class R>
__device__ __forceinline__ R pair_fs(R r2, R sig, R e24i, R sqrt_eps_j, R kqi, R qj, R& inv_r, R& s6) {
  inv_r = inv_sqrt_r(r2);
  const R inv_r2 = inv_r * inv_r;
  const R s2 = sig * sig * inv_r2;
  s6 = s2 * s2 * s2;
  const R u = s6 * fma_r(R(2.0f), s6, R(-1.0f));  // 2 s6^2 - s6
  const R cr = kqi * qj * inv_r;
  return fma_r(e24i * sqrt_eps_j, u, cr) * inv_r2;
}

// f -= fs * d, one rounding per component.
template <class R>
__device__ __forceinline__ void acc_pair(Acc<R>& f, R fs, R dx, R dy, R dz) {
  f.x = fma_r(-fs, dx, f.x);
  f.y = fma_r(-fs, dy, f.y);
  f.z = fma_r(-fs, dz, f.z);
}

// Sum over the 4 lanes of one atom (fixed butterfly: exact for int64,
// order-fixed for double).
__device__ __forceinline__ long long lane_sum(long long v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}
__device__ __forceinline__ double lane_sum(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}

// One ordinary pair, branch-free: force on i from j when r^2 lies in
// [0.01, cutoff^2), an exact zero otherwise.
template <class R>
__device__ __forceinline__ void pair_accumulate(const R4<R> pi, R kqi, R sig_i, R e24i, const R4<R> pj, R2<R> lj,
                                                R cut2, Acc<R>& f) {
  const R dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
  const R r2 = fma_r(dz, dz, fma_r(dy, dy, dx * dx));
  const bool in = r2 < cut2 && r2 >= R(kMinPairR2);
  R inv_r, s6;
  // outside [0.01, cutoff^2) the law may overflow or divide by zero; the
  // select below discards that value
  R fs = pair_fs<R>(r2, sig_i + lj.x, e24i, lj.y, kqi, pj.w, inv_r, s6);
  fs = in ? fs : R(0.0f);
  acc_pair<R>(f, fs, dx, dy, dz);
}

__device__ __forceinline__ void store_force(const Arena& A, int a, const Acc<float>& f) {
  const long long X = lane_sum(f.X), Y = lane_sum(f.Y), Z = lane_sum(f.Z);
  if ((threadIdx.x & 3) == 0) {
    const int64_t cap = A.atom_cap;
    A.f[a] = X;
    A.f[cap + a] = Y;
    A.f[2 * cap + a] = Z;
  }
}
__device__ __forceinline__ void store_force(const Arena& A, int a, const Acc<double>& f) {
  const double X = lane_sum(f.x), Y = lane_sum(f.y), Z = lane_sum(f.z);
  if ((threadIdx.x & 3) == 0) {
    const int64_t cap = A.atom_cap;
    A.f64[a] = X;
    A.f64[cap + a] = Y;
    A.f64[2 * cap + a] = Z;
  }
}

// ---- per-term contributions, as each member's gather adds them ----
//
// A term is evaluated once; member m's contribution is the value the member
// would add to its own force if it evaluated the term itself: for a bond
// -fm*r and +fm*r (r = x_j - x_i, fm = -2k(r - r0)/r), for an angle -(fm*d)
// at the ends and fm*(d_i + d_k) at the apex, for a torsion f1, s - f1,
// -s - f4 and f4 (the OpenMM torsion gradient), for an exception -(fs*d)
// seen from either member (d = x_partner - x_self, the same number negated).
template <class R>
struct TermOut {
  R x[4], y[4], z[4];
  double e;  // energy share of every member
};

template <class R>
__device__ __forceinline__ bool bond_out(const R4<R>* pos, const BondT b, TermOut<R>& o) {
  const R4<R> pi = pos[b.i], pj = pos[b.j];
  const R rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
  const R r = sqrt_r(rx * rx + ry * ry + rz * rz);
  if (r < R(1e-8f)) return false;
  const R dr = r - R(b.r0);
  const R fm = R(-2.0f) * R(b.k) * dr / r;
  const R sn = -fm;
  o.x[0] = sn * rx; o.y[0] = sn * ry; o.z[0] = sn * rz;
  o.x[1] = fm * rx; o.y[1] = fm * ry; o.z[1] = fm * rz;
  o.e = (double)b.k * (double)dr * (double)dr * 0.5;
  return true;
}

template <class R>
__device__ __forceinline__ bool angle_out(const R4<R>* pos, const AngleT a, TermOut<R>& o) {
  const R4<R> pi = pos[a.i], pj = pos[a.j], pk = pos[a.k];
  const R ax = pi.x - pj.x, ay = pi.y - pj.y, az = pi.z - pj.z;  // rij
  const R bx = pk.x - pj.x, by = pk.y - pj.y, bz = pk.z - pj.z;  // rkj
  const R la = sqrt_r(ax * ax + ay * ay + az * az);
  const R lb = sqrt_r(bx * bx + by * by + bz * bz);
  if (la < R(1e-8f) || lb < R(1e-8f)) return false;
  R c = (ax * bx + ay * by + az * bz) / (la * lb);
  c = max_r(R(-1.0f), min_r(R(1.0f), c));
  const R th = acos_r(c);
  const R dth = th - R(a.theta0);
  R sn = sqrt_r(R(1.0f) - c * c);
  if (sn < R(1e-8f)) sn = R(1e-8f);
  const R fm = R(-2.0f) * R(a.kf) * dth / sn;
  const R ia = R(1.0f) / la, ib = R(1.0f) / lb;
  const R dix = (bx * ib - c * ax * ia) * ia, diy = (by * ib - c * ay * ia) * ia, diz = (bz * ib - c * az * ia) * ia;
  const R dkx = (ax * ia - c * bx * ib) * ib, dky = (ay * ia - c * by * ib) * ib, dkz = (az * ia - c * bz * ib) * ib;
  o.x[0] = -(fm * dix); o.y[0] = -(fm * diy); o.z[0] = -(fm * diz);
  o.x[2] = -(fm * dkx); o.y[2] = -(fm * dky); o.z[2] = -(fm * dkz);
  o.x[1] = fm * (dix + dkx); o.y[1] = fm * (diy + dky); o.z[1] = fm * (diz + dkz);
  o.e = (double)a.kf * (double)dth * (double)dth * (1.0 / 3.0);
  return true;
}

// Periodic torsion U = k (1 + cos(n phi - delta)) / 4 with the OpenMM
// gradient (compute_dihedral_force, nhs_amber_fused.cu:525).  phi is not
// formed: cos phi = c0.c1 / (|c0||c1|) and, because c0 x c1 = v1 (v0.c1),
// sin phi = |v1| (v0.c1) / (|c0||c1|) with the reference's sign (phi < 0
// when v0.c1 < 0); cos and sin of n phi follow by the angle-addition
// recurrence and sin(n phi - delta) = sin(n phi) cos(delta) - cos(n phi)
// sin(delta) from cos(delta), sin(delta) computed once per term on the host.
// The reference takes phi through acosf/asinf and then sinf; the two agree to
// FP32 rounding.
template <class R>
__device__ __forceinline__ bool dihedral_out(const R4<R>* pos, const DihT d, TermOut<R>& o) {
  const R4<R> pi = pos[d.i], pj = pos[d.j], pk = pos[d.k], pl = pos[d.l];
  const R v0x = pi.x - pj.x, v0y = pi.y - pj.y, v0z = pi.z - pj.z;
  const R v1x = pk.x - pj.x, v1y = pk.y - pj.y, v1z = pk.z - pj.z;
  const R v2x = pk.x - pl.x, v2y = pk.y - pl.y, v2z = pk.z - pl.z;
  const R c0x = v0y * v1z - v0z * v1y, c0y = v0z * v1x - v0x * v1z, c0z = v0x * v1y - v0y * v1x;
  const R c1x = v1y * v2z - v1z * v2y, c1y = v1z * v2x - v1x * v2z, c1z = v1x * v2y - v1y * v2x;
  const R n1 = c0x * c0x + c0y * c0y + c0z * c0z;
  const R n2 = c1x * c1x + c1y * c1y + c1z * c1z;
  const R nb = v1x * v1x + v1y * v1y + v1z * v1z;
  if (n1 < R(1e-16f) || n2 < R(1e-16f) || nb < R(1e-16f)) return false;
  const R lbc = sqrt_r(nb);
  const R inv_n12 = R(1.0f) / sqrt_r(n1 * n2);
  R cp = (c0x * c1x + c0y * c1y + c0z * c1z) * inv_n12;
  R sp = lbc * (v0x * c1x + v0y * c1y + v0z * c1z) * inv_n12;
  cp = max_r(R(-1.0f), min_r(R(1.0f), cp));
  sp = max_r(R(-1.0f), min_r(R(1.0f), sp));
  // cos and sin of n phi (the lowering keeps 1 <= n <= kMaxPeriodicity)
  R cn = R(1.0f), sn = R(0.0f);
  for (int k = 0; k < d.n; ++k) {
    const R c2 = cn * cp - sn * sp;
    sn = sn * cp + cn * sp;
    cn = c2;
  }
  const R n = (R)d.n;
  const R dE = -R(d.kf) * n * (sn * R(d.cos_ph) - cn * R(d.sin_ph));
  const R inb = R(1.0f) / nb;
  const R ff0 = (-dE * lbc) / n1;
  const R ff1 = (v0x * v1x + v0y * v1y + v0z * v1z) * inb;
  const R ff2 = (v2x * v1x + v2y * v1y + v2z * v1z) * inb;
  const R ff3 = (dE * lbc) / n2;
  const R f1x = ff0 * c0x, f1y = ff0 * c0y, f1z = ff0 * c0z;
  const R f4x = ff3 * c1x, f4y = ff3 * c1y, f4z = ff3 * c1z;
  const R sx = ff1 * f1x - ff2 * f4x, sy = ff1 * f1y - ff2 * f4y, sz = ff1 * f1z - ff2 * f4z;
  o.x[0] = f1x; o.y[0] = f1y; o.z[0] = f1z;
  o.x[1] = sx - f1x; o.y[1] = sy - f1y; o.z[1] = sz - f1z;
  o.x[2] = -sx - f4x; o.y[2] = -sy - f4y; o.z[2] = -sz - f4z;
  o.x[3] = f4x; o.y[3] = f4y; o.z[3] = f4z;
  o.e = (double)d.kf * (1.0 + ((double)cn * (double)d.cos_ph + (double)sn * (double)d.sin_ph)) * 0.25;
  return true;
}

// exact exceptions: no cutoff, no shift (nhs_amber_fused.cu:3316-3467)
template <class R>
__device__ __forceinline__ bool exception_out(const R4<R>* pos, const ExcT e, TermOut<R>& o, bool& bad) {
  const R4<R> pi = pos[e.i], pj = pos[e.j];
  const R dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
  const R r2 = fma_r(dz, dz, fma_r(dy, dy, dx * dx));
  if (r2 < R(1e-8f)) {
    bad = true;
    return false;
  }
  R inv_r, s6;
  const R fs = pair_scalar<R>(r2, R(e.sig), R(e.eps), R(e.qq), inv_r, s6);
  const R px = fs * dx, py = fs * dy, pz = fs * dz;
  o.x[0] = -px; o.y[0] = -py; o.z[0] = -pz;
  o.x[1] = px; o.y[1] = py; o.z[1] = pz;
  o.e = (4.0 * (double)e.eps * ((double)s6 * (double)s6 - (double)s6) +
         (double)kCoulomb * (double)e.qq * (double)inv_r) * 0.5;
  return true;
}

// Ordinary pairs from cluster-pair tiles (FP32 complete-mode systems).  Warp
// w of the block owns i-cluster w (atoms a0 + 8w .. a0 + 8w + 7) and lane
// i + 8 jj evaluates pair (i, jj) of every tile in the i-cluster's list, so a
// tile's four j atoms are read once for all eight i atoms (a 64-byte line
// shared by the warp) and the list costs 8 bytes per 32 pair slots.  A
// tile whose pairs all lie outside the cutoff costs only the distance test
// (warp vote).  The inclusion test (list bit, r^2 in [0.01, cutoff^2)) and
// the pair law are the row path's; lane jj sums FP32 over its pairs of 32
// consecutive tiles, then accumulates in int64, and an atom's four lanes are
// summed exactly, so the force depends only on the system's own tile list.
template <bool kEnergy>
__device__ __forceinline__ void force_tiles(const Arena& A, int64_t n_span, int s0, const SysDev* Sp, int64_t a0,
                                            int tid, const float* slot_x, const float* slot_y, const float* slot_z,
                                            const double* slot_e, const int* s_base, const int* s_nb,
                                            const int* s_na, const int* s_nd) {
  const int lane = tid & 31, w = tid >> 5;
  const int64_t c0 = a0 + (w << 3);  // the warp's i-cluster
  if (c0 >= n_span || A.atom_sys[c0] != s0) return;  // whole warp
  const int ga = (w << 3) + (lane & 7), q = lane >> 3;
  const int64_t a64 = a0 + ga;
  const bool mine = a64 < n_span && A.atom_sys[a64] == s0;
  const int a = mine ? (int)a64 : (int)c0;  // lanes past the system's end stand in with the cluster's first atom
  const float cut2 = Sp->cut2;
  Acc<float> f{};
  double eb = 0.0, ea = 0.0, ed = 0.0, ex = 0.0, en = 0.0;
  if (mine) {
    const int base = s_base[ga], nb = s_nb[ga], na = s_na[ga], nd = s_nd[ga];
    for (int t = q; t < nb; t += kLanes) {
      f.x += slot_x[base + t];
      f.y += slot_y[base + t];
      f.z += slot_z[base + t];
      if (kEnergy) eb += slot_e[base + t];
    }
    for (int t = q; t < na; t += kLanes) {
      const int sl = base + nb + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ea += slot_e[sl];
    }
    for (int t = q; t < nd; t += kLanes) {
      const int sl = base + nb + na + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ed += slot_e[sl];
    }
    f.flush();
    const int ne = A.ex_idx[a].y;
    for (int t = q; t < ne; t += kLanes) {
      const int sl = base + nb + na + nd + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ex += slot_e[sl];
    }
    f.flush();
  }
  const float4 pi = A.pos[a];
  const float2 li = A.lj[a];
  const float qi = pi.w;
  const int64_t g = c0 >> 3;
  const int nt = A.ntile[g];
  const int2* tl = A.tiles + g * kTileCap;
  const unsigned lanebit = 1u << lane;
  float inv_rc = 0.0f;
  if (kEnergy) inv_rc = rsqrtf(cut2);
  for (int t0 = 0; t0 < nt; t0 += 32) {
    const int2 e = t0 + lane < nt ? __ldg(tl + t0 + lane) : make_int2(0, 0);
    const int m = min(32, nt - t0);
    for (int u = 0; u < m; ++u) {
      const int jc = __shfl_sync(0xffffffffu, e.x, u);
      const unsigned bits = (unsigned)__shfl_sync(0xffffffffu, e.y, u);
      const int j = (jc << 2) + q;
      const float4 pj = __ldg(A.pos + j);
      const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const bool in = (bits & lanebit) != 0u && r2 < cut2 && r2 >= kMinPairR2;
      if (__any_sync(0xffffffffu, in)) {
        // lanes outside the list or the cutoff add an exact zero (the j atoms
        // past a system's end hold finite positions: admission zeroes them)
        const float2 lj = __ldg(A.lj + j);
        const float sig = li.x + lj.x, eps = li.y * lj.y, qq = qi * pj.w;
        float inv_r, s6;
        float fs = pair_scalar<float>(fmaxf(r2, kMinPairR2), sig, eps, qq, inv_r, s6);
        fs = in ? fs : 0.0f;
        acc_pair<float>(f, fs, dx, dy, dz);
        if (kEnergy && in) {
          const float sc2 = sig * sig * inv_rc * inv_rc;
          const float sc6 = sc2 * sc2 * sc2;
          const double v = 4.0 * (double)eps * (((double)s6 * (double)s6 - (double)s6) -
                                                ((double)sc6 * (double)sc6 - (double)sc6)) +
                           (double)kCoulomb * (double)qq * ((double)inv_r - (double)inv_rc);
          en += v * 0.5;
        }
      }
    }
    f.flush();
  }
  long long X = f.X, Y = f.Y, Z = f.Z;
#pragma unroll
  for (int o = 8; o <= 16; o <<= 1) {
    X += __shfl_xor_sync(0xffffffffu, X, o);
    Y += __shfl_xor_sync(0xffffffffu, Y, o);
    Z += __shfl_xor_sync(0xffffffffu, Z, o);
  }
  if (kEnergy) {
#pragma unroll
    for (int o = 8; o <= 16; o <<= 1) {
      eb += __shfl_xor_sync(0xffffffffu, eb, o);
      ea += __shfl_xor_sync(0xffffffffu, ea, o);
      ed += __shfl_xor_sync(0xffffffffu, ed, o);
      ex += __shfl_xor_sync(0xffffffffu, ex, o);
      en += __shfl_xor_sync(0xffffffffu, en, o);
    }
  }
  if (mine && q == 0) {
    const int64_t cap = A.atom_cap;
    A.f[a] = X;
    A.f[cap + a] = Y;
    A.f[2 * cap + a] = Z;
    if (kEnergy) {
      A.pe[a] = eb;
      A.pe[cap + a] = ea;
      A.pe[2 * cap + a] = ed;
      A.pe[3 * cap + a] = ex;
      A.pe[4 * cap + a] = en;
    }
  }
}

// One force block = one 32-atom group, four lanes per atom.
//   1. The block evaluates every bonded term and exception pair with a member
//      in the group once (one thread per term), and drops each member's
//      contribution into a shared-memory slot: the member's incidence entries
//      of each kind, in the order the member lists them.
//   2. Lane q of an atom sums the slots of its entries with index ≡ q (mod 4),
//      bonded kinds first, then exceptions, then its row entries ≡ q (mod 4).
// Each lane keeps FP32 partial sums over at most 32 of its entries and
// accumulates them in int64; the lanes' int64 totals are then summed exactly.
// The decomposition depends only on the atom's own lists, so an atom's force
// is identical whatever batch it is computed in.  The reference recomputes
// each term for every member atom (nhs_amber_fused.cu:3002-3090); evaluating
// it once per group gives each member the same contribution.
//
// A block holds kG such groups (128 threads each, consecutive groups); the
// groups share nothing but the block's barriers, so kG changes the launch
// shape, never the results.
template <class R, bool kEnergy, int kMinBlocks, int kG, int kPf>
__global__ void __launch_bounds__(128 * kG, kMinBlocks) k_force(Arena A, int64_t n_span, int sel, int cap) {
  // a pass over the systems the preceding control kernel rebuilt has nothing
  // to do when the row builder before it found the queue empty (a refresh
  // after an upload that moved no position)
  if (sel == kSelRebuilding && A.work_ctl[3] == 0) return;
  // the row builder that ran before this launch consumed the rebuild queue
  // (the branch-B launch of an overlapped step may run beside that builder)
  if (sel != kSelBranchB && blockIdx.x == 0 && threadIdx.x == 0) {
    A.work_ctl[0] = 0;
    A.work_ctl[1] = 0;
    A.work_ctl[2] = 0;
  }
  extern __shared__ __align__(16) unsigned char force_smem[];
  __shared__ int s_base_g[kG][kForceGroup], s_nb_g[kG][kForceGroup], s_na_g[kG][kForceGroup],
      s_nd_g[kG][kForceGroup];
  const int sub = threadIdx.x >> 7;  // the block's group this thread works on
  const int tid = threadIdx.x & 127, q = tid & 3;
  int* s_base = s_base_g[sub];
  int* s_nb = s_nb_g[sub];
  int* s_na = s_na_g[sub];
  int* s_nd = s_nd_g[sub];
  const int64_t gi = (int64_t)blockIdx.x * kG + sub;
  const int64_t a0 = gi * kForceGroup;
  // a group with nothing to do skips its work but still meets the barriers
  bool skip = a0 >= n_span;
  const int s0 = skip ? -1 : A.atom_sys[a0];
  skip = skip || s0 < 0;
  const SysDev* Sp = skip ? nullptr : &A.sys[s0];
  if (!skip) {
    skip = !Sp->active || (sel == kSelRebuilding && !Sp->rebuilding) || (sel == kSelBranchA && !Sp->branch_a) ||
           (sel == kSelBranchB && Sp->branch_a);
  }
  // a block of one group has no partner group to meet at the barriers
  if constexpr (kG == 1) {
    if (skip) return;
  }
  const size_t slot_bytes = (size_t)cap * (3 * sizeof(R) + (kEnergy ? sizeof(double) : 0));
  R* slot_x = reinterpret_cast<R*>(force_smem + sub * slot_bytes);
  R* slot_y = slot_x + cap;
  R* slot_z = slot_y + cap;
  double* slot_e = reinterpret_cast<double*>(slot_z + cap);
  // ---- slot layout of the group's atoms ----
  if (!skip && tid < kForceGroup) {
    const int64_t b = a0 + tid;
    int nb = 0, na = 0, nd = 0, ne = 0;
    if (b < n_span && A.atom_sys[b] == s0) {
      const Incidence I = A.inc[b];
      nb = I.counts & 0xff;
      na = (I.counts >> 8) & 0xff;
      nd = (I.counts >> 16) & 0xff;
      ne = A.ex_idx[b].y;
    }
    const int tot = nb + na + nd + ne;
    int incl = tot;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (tid >= o) incl += v;
    }
    s_base[tid] = incl - tot;
    s_nb[tid] = nb;
    s_na[tid] = na;
    s_nd[tid] = nd;
  }
  __syncthreads();
  const R4<R>* pos = positions(A, R(0));
  // ---- every term with a member in the group, once ----
  const int2 gr = skip ? make_int2(0, 0) : A.grp[gi];
  bool bad = false;
  for (int r = tid; r < gr.y; r += 128) {
    const int ref = A.grp_refs[gr.x + r];
    const int kind = ref >> 29, t = ref & ((1 << 29) - 1);
    TermOut<R> o;
    int mem[4], pp[4], nm, koff;  // koff: 0 bonds, 1 angles, 2 torsions, 3 exceptions
    bool ok;
    if (kind == kRefBond) {
      const BondT b = A.bonds[t];
      ok = bond_out<R>(pos, b, o);
      nm = 2; mem[0] = b.i; mem[1] = b.j; pp[0] = b.pos & 0xffff; pp[1] = b.pos >> 16;
    } else if (kind == kRefAngle) {
      const AngleT g = A.angles[t];
      ok = angle_out<R>(pos, g, o);
      nm = 3; mem[0] = g.i; mem[1] = g.j; mem[2] = g.k;
      pp[0] = g.pos & 1023; pp[1] = (g.pos >> 10) & 1023; pp[2] = (g.pos >> 20) & 1023;
    } else if (kind == kRefDih) {
      const DihT d = A.dihs[t];
      ok = dihedral_out<R>(pos, d, o);
      nm = 4; mem[0] = d.i; mem[1] = d.j; mem[2] = d.k; mem[3] = d.l;
      pp[0] = d.pos & 255; pp[1] = (d.pos >> 8) & 255; pp[2] = (d.pos >> 16) & 255; pp[3] = (d.pos >> 24) & 255;
    } else {
      const ExcT e = A.exc[t];
      ok = exception_out<R>(pos, e, o, bad);
      nm = 2; mem[0] = e.i; mem[1] = e.j; pp[0] = e.pos & 0xffff; pp[1] = e.pos >> 16;
    }
    koff = kind;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (m >= nm) break;
      const int li = (int)(mem[m] - a0);
      if (li < 0 || li >= kForceGroup) continue;
      const int off = koff == 0 ? 0 : koff == 1 ? s_nb[li] : koff == 2 ? s_nb[li] + s_na[li]
                                                               : s_nb[li] + s_na[li] + s_nd[li];
      const int sl = s_base[li] + off + pp[m];
      if (sl >= cap) {  // cannot happen: cap covers the fullest group
        bad = true;
        continue;
      }
      slot_x[sl] = ok ? o.x[m] : R(0.0f);
      slot_y[sl] = ok ? o.y[m] : R(0.0f);
      slot_z[sl] = ok ? o.z[m] : R(0.0f);
      if (kEnergy) slot_e[sl] = ok ? o.e : 0.0;
    }
  }
  if (bad) atomicOr(&A.sys[s0].status, kStNonfinite);
  __syncthreads();
  if (skip) return;
  if constexpr (sizeof(R) == 4) {
    if (uses_tiles(A, *Sp)) {
      force_tiles<kEnergy>(A, n_span, s0, Sp, a0, tid, reinterpret_cast<const float*>(slot_x),
                           reinterpret_cast<const float*>(slot_y), reinterpret_cast<const float*>(slot_z), slot_e,
                           s_base, s_nb, s_na, s_nd);
      return;
    }
  }
  const int ga = tid >> 2;  // the thread's atom within the group
  const int64_t a64 = a0 + ga;
  if (a64 >= n_span || A.atom_sys[a64] != s0) return;
  const int a = (int)a64;
  const R cut2 = R(Sp->cut2);
  Acc<R> f{};
  double eb = 0.0, ea = 0.0, ed = 0.0, ex = 0.0, en = 0.0;
  {
    const int base = s_base[ga], nb = s_nb[ga], na = s_na[ga], nd = s_nd[ga];
    for (int t = q; t < nb; t += kLanes) {
      f.x += slot_x[base + t];
      f.y += slot_y[base + t];
      f.z += slot_z[base + t];
      if (kEnergy) eb += slot_e[base + t];
    }
    for (int t = q; t < na; t += kLanes) {
      const int sl = base + nb + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ea += slot_e[sl];
    }
    for (int t = q; t < nd; t += kLanes) {
      const int sl = base + nb + na + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ed += slot_e[sl];
    }
    f.flush();
    const int ne = A.ex_idx[a].y;
    for (int t = q; t < ne; t += kLanes) {
      const int sl = base + nb + na + nd + t;
      f.x += slot_x[sl];
      f.y += slot_y[sl];
      f.z += slot_z[sl];
      if (kEnergy) ex += slot_e[sl];
    }
    f.flush();
  }
  const R4<R> pi = pos[a];

  // ordinary pairs: lane q walks entries q, q+4, ... of the tiled row
  const R2<R>* ljp = lj_params(A, R(0));
  const R2<R> li = ljp[a];
  const R qi = pi.w;
  const R kqi = R(kCoulomb) * qi, e24i = R(24.0f) * li.y;
  const int n = A.nnbr[a];
  const int* row = A.nbr + nbr_index(a, q);  // entry 4t+q is at row[128 (t/4) + t%4]
  R inv_rc = R(0.0f);
  if (kEnergy) inv_rc = inv_sqrt_r(cut2);
  const int mine = n > q ? (n - q + kLanes - 1) / kLanes : 0;
  if constexpr (!kEnergy) {
    // Force-only path: entries are processed four at a time with every load
    // issued before any arithmetic, and the cutoff is a select instead of a
    // branch, so a lane keeps several gathers in flight and lanes never
    // diverge.  Pairs outside the cutoff contribute an exact zero, so the sum
    // is the same sequence of additions as a branching loop.
    // The row indices of the next four entries (one int4) are loaded while
    // the current four are gathered and evaluated.  Partial sums flush after
    // every 32 of the lane's entries, as in a loop over 32-entry chunks.
    const int m4 = mine & ~3;
    const int4* row4 = reinterpret_cast<const int4*>(row);  // block t/4 of the lane at row4[32 (t/4)]
    constexpr int kL2 = kPf;  // row block requested into L2 this many iterations ahead
    int4 jn = m4 > 0 ? __ldg(row4) : make_int4(0, 0, 0, 0);
    for (int t = 0; t < m4; t += 4) {
      const int j[4] = {jn.x, jn.y, jn.z, jn.w};
      R4<R> pj[4];
      R2<R> lj[4];
      if (t + 4 < m4) jn = __ldg(row4 + (int64_t)(t + 4) * 8);
      // the row block kL2 iterations ahead is requested into L2 now (inside
      // the lane's own row storage; a prefetch moves no data into registers
      // and changes no result)
      if (kL2 > 0 && t + 4 * kL2 < m4) {
        const int4* ahead = row4 + (int64_t)(t + 4 * kL2) * 8;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(ahead));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        pj[u] = ldg_r4(pos + j[u]);
        lj[u] = __ldg(ljp + j[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) pair_accumulate<R>(pi, kqi, li.x, e24i, pj[u], lj[u], cut2, f);
      if (((t + 4) & 31) == 0) f.flush();
    }
    for (int t = m4; t < mine; ++t) {
      const int j = __ldg(row + (int64_t)(t >> 2) * 128 + (t & 3));
      pair_accumulate<R>(pi, kqi, li.x, e24i, ldg_r4(pos + j), __ldg(ljp + j), cut2, f);
    }
    f.flush();
  } else
    for (int t0 = 0; t0 < mine; t0 += 32) {
      const int t1 = min(mine, t0 + 32);
#pragma unroll 4
      for (int t = t0; t < t1; ++t) {
        const int j = __ldg(row + (int64_t)(t >> 2) * 128 + (t & 3));
        const R4<R> pj = ldg_r4(pos + j);
        const R dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const R r2 = fma_r(dz, dz, fma_r(dy, dy, dx * dx));
        if (r2 < cut2 && r2 >= R(kMinPairR2)) {
          const R2<R> lj = __ldg(ljp + j);
          const R sig = li.x + lj.x, eps = li.y * lj.y, qq = qi * pj.w;
          R inv_r, s6;
          const R fs = pair_fs<R>(r2, sig, e24i, lj.y, kqi, pj.w, inv_r, s6);
          acc_pair<R>(f, fs, dx, dy, dz);
          if (kEnergy) {
            const R sc2 = sig * sig * inv_rc * inv_rc;
            const R sc6 = sc2 * sc2 * sc2;
            const double v = 4.0 * (double)eps * (((double)s6 * (double)s6 - (double)s6) -
                                                  ((double)sc6 * (double)sc6 - (double)sc6)) +
                             (double)kCoulomb * (double)qq * ((double)inv_r - (double)inv_rc);
            en += v * 0.5;
          }
        }
      }
      f.flush();
    }
  store_force(A, a, f);
  if (kEnergy) {
    eb = lane_sum(eb);
    ea = lane_sum(ea);
    ed = lane_sum(ed);
    ex = lane_sum(ex);
    en = lane_sum(en);
    if (q == 0) {
      const int64_t cap = A.atom_cap;
      A.pe[a] = eb;
      A.pe[cap + a] = ea;
      A.pe[2 * cap + a] = ed;
      A.pe[3 * cap + a] = ex;
      A.pe[4 * cap + a] = en;
    }
  }
}

// Launch shapes of the force-only kernel the autotuner chooses from: atoms
// per block (32 or 64: one or two force groups) and the minimum resident
// blocks per SM handed to the register allocator.  The shape changes neither
// the per-atom decomposition nor the results.
// Variants 7-13 repeat 0-6 with the row indices requested into L2 four
// iterations (16 entries per atom) ahead.
struct ForceShape {
  int block, min_blocks, prefetch;
};
static const ForceShape kForceShapes[] = {{128, 1, 0}, {128, 8, 0}, {128, 10, 0}, {128, 12, 0},
                                          {256, 4, 0}, {256, 5, 0}, {256, 6, 0},
                                          {128, 1, 4}, {128, 8, 4}, {128, 10, 4}, {128, 12, 4},
                                          {256, 4, 4}, {256, 5, 4}, {256, 6, 4}};

int force_variant_count() { return (int)(sizeof(kForceShapes) / sizeof(kForceShapes[0])); }

void force_variant_shape(int v, int* block, int* min_blocks) {
  *block = kForceShapes[v].block;
  *min_blocks = kForceShapes[v].min_blocks;
}

int force_variant_prefetch(int v) { return kForceShapes[v].prefetch; }

template <class R, bool kEnergy, int kMinBlocks, int kG = 1, int kPf = 0>
static void force_launch(const Arena& A, int64_t n, int ob, int cap, cudaStream_t st) {
  const size_t smem = (size_t)kG * cap * (3 * sizeof(R) + (kEnergy ? sizeof(double) : 0));
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_force<R, kEnergy, kMinBlocks, kG, kPf>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)((size_t)kG * kMaxGroupSlots * (3 * sizeof(R) + sizeof(double))));
    attr = true;
  }
  const int64_t groups = (n + kForceGroup - 1) / kForceGroup;
  const unsigned blocks = (unsigned)((groups + kG - 1) / kG);
  k_force<R, kEnergy, kMinBlocks, kG, kPf><<<blocks, 128 * kG, smem, st>>>(A, n, ob, cap);
}

void launch_force(const Arena& A, int64_t n_atoms_span, bool energy, cudaStream_t st, int sel, int variant,
                  int group_slots) {
  if (n_atoms_span <= 0) return;
  const int ob = sel;
  const int cap = (std::max(group_slots, 1) + 7) & ~7;  // keeps the FP64 energy plane 8-byte aligned
  if (A.fp64) {
    if (energy)
      force_launch<double, true, 1>(A, n_atoms_span, ob, cap, st);
    else
      force_launch<double, false, 1>(A, n_atoms_span, ob, cap, st);
    return;
  }
  if (energy) {
    force_launch<float, true, 1>(A, n_atoms_span, ob, cap, st);
    return;
  }
  switch (variant) {
    case 1: force_launch<float, false, 8>(A, n_atoms_span, ob, cap, st); break;
    case 2: force_launch<float, false, 10>(A, n_atoms_span, ob, cap, st); break;
    case 3: force_launch<float, false, 12>(A, n_atoms_span, ob, cap, st); break;
    case 4: force_launch<float, false, 4, 2>(A, n_atoms_span, ob, cap, st); break;
    case 5: force_launch<float, false, 5, 2>(A, n_atoms_span, ob, cap, st); break;
    case 6: force_launch<float, false, 6, 2>(A, n_atoms_span, ob, cap, st); break;
    case 7: force_launch<float, false, 1, 1, 4>(A, n_atoms_span, ob, cap, st); break;
    case 8: force_launch<float, false, 8, 1, 4>(A, n_atoms_span, ob, cap, st); break;
    case 9: force_launch<float, false, 10, 1, 4>(A, n_atoms_span, ob, cap, st); break;
    case 10: force_launch<float, false, 12, 1, 4>(A, n_atoms_span, ob, cap, st); break;
    case 11: force_launch<float, false, 4, 2, 4>(A, n_atoms_span, ob, cap, st); break;
    case 12: force_launch<float, false, 5, 2, 4>(A, n_atoms_span, ob, cap, st); break;
    case 13: force_launch<float, false, 6, 2, 4>(A, n_atoms_span, ob, cap, st); break;
    default: force_launch<float, false, 1>(A, n_atoms_span, ob, cap, st); break;
  }
}

}  // namespace pq
