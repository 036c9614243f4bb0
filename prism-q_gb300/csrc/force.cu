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
//   * neighbour rows are interleaved by 8-atom group so a warp's index loads
//     are one 128-byte line per k, and exception pairs are already excluded
//     from the rows (no per-neighbour 1-4 scan);
//   * partial sums are FP32 over at most 32 pairs and then accumulated in
//     int64 fixed point at 2^-32 kcal/mol/Å, so the force of an atom is a
//     deterministic function of its own row alone;
//   * energies are computed only by the energy variant (FP64 per-atom planes).
#include "pq_common.cuh"
#include "pq_device.cuh"

namespace pq {

struct Acc {
  float x, y, z;
  long long X, Y, Z;
  __device__ __forceinline__ void flush() {
    X += f2fixed(x);
    Y += f2fixed(y);
    Z += f2fixed(z);
    x = y = z = 0.0f;
  }
};

// ---- bonded laws (FP32) ----

__device__ __forceinline__ void bond_term(const float4* pos, const BondT b, int p, Acc& f, double* e) {
  const float4 pi = pos[b.i], pj = pos[b.j];
  const float rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
  const float r = sqrtf(rx * rx + ry * ry + rz * rz);
  if (r < 1e-8f) return;
  const float dr = r - b.r0;
  const float fm = -2.0f * b.k * dr / r;
  const float s = p == 0 ? -fm : fm;  // fi -= f, fj += f
  f.x += s * rx;
  f.y += s * ry;
  f.z += s * rz;
  if (e) *e += (double)b.k * (double)dr * (double)dr * 0.5;
}

__device__ __forceinline__ void angle_term(const float4* pos, const AngleT a, int p, Acc& f, double* e) {
  const float4 pi = pos[a.i], pj = pos[a.j], pk = pos[a.k];
  const float ax = pi.x - pj.x, ay = pi.y - pj.y, az = pi.z - pj.z;  // rij
  const float bx = pk.x - pj.x, by = pk.y - pj.y, bz = pk.z - pj.z;  // rkj
  const float la = sqrtf(ax * ax + ay * ay + az * az);
  const float lb = sqrtf(bx * bx + by * by + bz * bz);
  if (la < 1e-8f || lb < 1e-8f) return;
  float c = (ax * bx + ay * by + az * bz) / (la * lb);
  c = fmaxf(-1.0f, fminf(1.0f, c));
  const float th = acosf(c);
  const float dth = th - a.theta0;
  float sn = sqrtf(1.0f - c * c);
  if (sn < 1e-8f) sn = 1e-8f;
  const float fm = -2.0f * a.kf * dth / sn;
  const float ia = 1.0f / la, ib = 1.0f / lb;
  const float dix = (bx * ib - c * ax * ia) * ia, diy = (by * ib - c * ay * ia) * ia,
              diz = (bz * ib - c * az * ia) * ia;
  const float dkx = (ax * ia - c * bx * ib) * ib, dky = (ay * ia - c * by * ib) * ib,
              dkz = (az * ia - c * bz * ib) * ib;
  if (p == 0) {
    f.x -= fm * dix;
    f.y -= fm * diy;
    f.z -= fm * diz;
  } else if (p == 2) {
    f.x -= fm * dkx;
    f.y -= fm * dky;
    f.z -= fm * dkz;
  } else {
    f.x += fm * (dix + dkx);
    f.y += fm * (diy + dky);
    f.z += fm * (diz + dkz);
  }
  if (e) *e += (double)a.kf * (double)dth * (double)dth * (1.0 / 3.0);
}

__device__ __forceinline__ void dihedral_term(const float4* pos, const DihT d, int p, Acc& f, double* e) {
  const float4 pi = pos[d.i], pj = pos[d.j], pk = pos[d.k], pl = pos[d.l];
  const float v0x = pi.x - pj.x, v0y = pi.y - pj.y, v0z = pi.z - pj.z;
  const float v1x = pk.x - pj.x, v1y = pk.y - pj.y, v1z = pk.z - pj.z;
  const float v2x = pk.x - pl.x, v2y = pk.y - pl.y, v2z = pk.z - pl.z;
  const float c0x = v0y * v1z - v0z * v1y, c0y = v0z * v1x - v0x * v1z, c0z = v0x * v1y - v0y * v1x;
  const float c1x = v1y * v2z - v1z * v2y, c1y = v1z * v2x - v1x * v2z, c1z = v1x * v2y - v1y * v2x;
  const float n1 = c0x * c0x + c0y * c0y + c0z * c0z;
  const float n2 = c1x * c1x + c1y * c1y + c1z * c1z;
  const float nb = v1x * v1x + v1y * v1y + v1z * v1z;
  if (n1 < 1e-16f || n2 < 1e-16f || nb < 1e-16f) return;
  const float lbc = sqrtf(nb);
  float cp = (c0x * c1x + c0y * c1y + c0z * c1z) / sqrtf(n1 * n2);
  cp = fmaxf(-1.0f, fminf(1.0f, cp));
  float phi;
  if (cp > 0.99f || cp < -0.99f) {
    const float xx = c0y * c1z - c0z * c1y, xy = c0z * c1x - c0x * c1z, xz = c0x * c1y - c0y * c1x;
    float s2 = (xx * xx + xy * xy + xz * xz) / (n1 * n2);
    s2 = fmaxf(0.0f, fminf(1.0f, s2));
    phi = asinf(sqrtf(s2));
    if (cp < 0.0f) phi = 3.14159265358979323846f - phi;
  } else {
    phi = acosf(cp);
  }
  if (v0x * c1x + v0y * c1y + v0z * c1z < 0.0f) phi = -phi;
  const float n = (float)d.n;
  const float dE = -d.kf * n * sinf(n * phi - d.phase);
  const float inb = 1.0f / nb;
  const float ff0 = (-dE * lbc) / n1;
  const float ff1 = (v0x * v1x + v0y * v1y + v0z * v1z) * inb;
  const float ff2 = (v2x * v1x + v2y * v1y + v2z * v1z) * inb;
  const float ff3 = (dE * lbc) / n2;
  const float f1x = ff0 * c0x, f1y = ff0 * c0y, f1z = ff0 * c0z;
  const float f4x = ff3 * c1x, f4y = ff3 * c1y, f4z = ff3 * c1z;
  const float sx = ff1 * f1x - ff2 * f4x, sy = ff1 * f1y - ff2 * f4y, sz = ff1 * f1z - ff2 * f4z;
  switch (p) {
    case 0: f.x += f1x; f.y += f1y; f.z += f1z; break;
    case 1: f.x += sx - f1x; f.y += sy - f1y; f.z += sz - f1z; break;
    case 2: f.x += -sx - f4x; f.y += -sy - f4y; f.z += -sz - f4z; break;
    default: f.x += f4x; f.y += f4y; f.z += f4z; break;
  }
  if (e) *e += (double)d.kf * (1.0 + cos((double)n * (double)phi - (double)d.phase)) * 0.25;
}

// ---- pair law: force on i from j (d = xj - xi), LJ + Coulomb ----
__device__ __forceinline__ float pair_scalar(float r2, float sig, float eps, float qq, float& inv_r,
                                             float& s6) {
  inv_r = rsqrtf(r2);
  const float inv_r2 = inv_r * inv_r;
  const float s2 = sig * sig * inv_r2;
  s6 = s2 * s2 * s2;
  const float flj = 24.0f * eps * inv_r2 * (2.0f * s6 * s6 - s6);
  const float fc = kCoulomb * qq * inv_r2 * inv_r;
  return flj + fc;
}

// Sum an int64 over the 4 lanes of one atom (fixed butterfly: exact, order-free).
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

// Four lanes per atom: lane q takes bonded terms, exceptions and row entries
// with index ≡ q (mod 4).  Each lane keeps FP32 partial sums over at most 32 of
// its entries and accumulates them in int64; the lanes' int64 totals are then
// summed exactly.  The decomposition depends only on the atom's own lists, so
// an atom's force is identical whatever batch it is computed in.
// One ordinary pair, branch-free: force on i from j when r^2 lies in
// [0.01, cutoff^2), an exact zero otherwise.
__device__ __forceinline__ void pair_accumulate(const float4 pi, float qi, float2 li, const float4 pj, float2 lj,
                                                float cut2, Acc& f) {
  const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
  const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  const bool in = r2 < cut2 && r2 >= kMinPairR2;
  const float sig = li.x + lj.x, eps = li.y * lj.y, qq = qi * pj.w;
  float inv_r, s6;
  float fs = pair_scalar(fmaxf(r2, kMinPairR2), sig, eps, qq, inv_r, s6);
  fs = in ? fs : 0.0f;
  f.x -= fs * dx;
  f.y -= fs * dy;
  f.z -= fs * dz;
}

template <bool kEnergy, int kBlock, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_force(Arena A, int64_t n_span, int only_rebuilt) {
  // the row builder that ran before this launch consumed the rebuild queue
  if (blockIdx.x == 0 && threadIdx.x == 0) A.work_ctl[0] = 0;
  const int64_t a64 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int q = threadIdx.x & 3;
  bool live = a64 < n_span;
  const int a = live ? (int)a64 : 0;
  const int s = live ? A.atom_sys[a] : -1;
  live = live && s >= 0;
  const SysDev* Sp = live ? &A.sys[s] : nullptr;
  live = live && Sp->active && (!only_rebuilt || Sp->rebuilding);
  // all four lanes of an atom share `live`; whole quads leave together
  if (!live) return;
  const float cut2 = Sp->cut2;
  const float4* pos = A.pos;
  Acc f{0.f, 0.f, 0.f, 0, 0, 0};
  double eb = 0.0, ea = 0.0, ed = 0.0, ex = 0.0, en = 0.0;

  const Incidence I = A.inc[a];
  const int nb = I.counts & 0xff, na = (I.counts >> 8) & 0xff, nd = (I.counts >> 16) & 0xff;
  for (int t = q; t < nb; t += kLanes) {
    const int ent = A.inc_list[I.b_beg + t];
    bond_term(pos, A.bonds[ent >> 2], ent & 3, f, kEnergy ? &eb : nullptr);
  }
  for (int t = q; t < na; t += kLanes) {
    const int ent = A.inc_list[I.a_beg + t];
    angle_term(pos, A.angles[ent >> 2], ent & 3, f, kEnergy ? &ea : nullptr);
  }
  for (int t = q; t < nd; t += kLanes) {
    const int ent = A.inc_list[I.d_beg + t];
    dihedral_term(pos, A.dihs[ent >> 2], ent & 3, f, kEnergy ? &ed : nullptr);
  }
  f.flush();

  const float4 pi = pos[a];
  // exact exceptions: no cutoff, no shift (nhs_amber_fused.cu:3316-3467)
  const int2 xr = A.ex_idx[a];
  for (int t = q; t < xr.y; t += kLanes) {
    const int j = A.ex_partner[xr.x + t];
    const float4 par = A.ex_par[xr.x + t];
    const float4 pj = pos[j];
    const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    if (r2 < 1e-8f) {
      atomicOr(&A.sys[s].status, kStNonfinite);
      continue;
    }
    float inv_r, s6;
    const float fs = pair_scalar(r2, par.y, par.z, par.x, inv_r, s6);
    f.x -= fs * dx;
    f.y -= fs * dy;
    f.z -= fs * dz;
    if (kEnergy) {
      const double v = 4.0 * (double)par.z * ((double)s6 * (double)s6 - (double)s6) +
                       (double)kCoulomb * (double)par.x * (double)inv_r;
      ex += v * 0.5;
    }
  }
  f.flush();

  // ordinary pairs: lane q walks entries q, q+4, ... of the tiled row
  const float2 li = A.lj[a];
  const float qi = pi.w;
  const int n = A.nnbr[a];
  const int* row = A.nbr + nbr_index(a, q);  // entry 4t+q is at row[32 t]
  float inv_rc = 0.f;
  if (kEnergy) inv_rc = rsqrtf(cut2);
  const int mine = n > q ? (n - q + kLanes - 1) / kLanes : 0;
  if constexpr (!kEnergy) {
    // Force-only path: entries are processed four at a time with every load
    // issued before any arithmetic, and the cutoff is a select instead of a
    // branch, so a lane keeps several gathers in flight and lanes never
    // diverge.  Pairs outside the cutoff contribute an exact zero, so the sum
    // is the same sequence of additions as a branching loop.
    for (int t0 = 0; t0 < mine; t0 += 32) {
      const int t1 = min(mine, t0 + 32);
      int t = t0;
      for (; t + 4 <= t1; t += 4) {
        int j[4];
        float4 pj[4];
        float2 lj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) j[u] = __ldg(row + (int64_t)(t + u) * 32);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          pj[u] = __ldg(pos + j[u]);
          lj[u] = __ldg(A.lj + j[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) pair_accumulate(pi, qi, li, pj[u], lj[u], cut2, f);
      }
      for (; t < t1; ++t) {
        const int j = __ldg(row + (int64_t)t * 32);
        pair_accumulate(pi, qi, li, __ldg(pos + j), __ldg(A.lj + j), cut2, f);
      }
      f.flush();
    }
  } else
  for (int t0 = 0; t0 < mine; t0 += 32) {
    const int t1 = min(mine, t0 + 32);
#pragma unroll 4
    for (int t = t0; t < t1; ++t) {
      const int j = __ldg(row + (int64_t)t * 32);
      const float4 pj = __ldg(pos + j);
      const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      if (r2 < cut2 && r2 >= kMinPairR2) {
        const float2 lj = __ldg(A.lj + j);
        const float sig = li.x + lj.x, eps = li.y * lj.y, qq = qi * pj.w;
        float inv_r, s6;
        const float fs = pair_scalar(r2, sig, eps, qq, inv_r, s6);
        f.x -= fs * dx;
        f.y -= fs * dy;
        f.z -= fs * dz;
        if (kEnergy) {
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
  const long long X = lane_sum(f.X), Y = lane_sum(f.Y), Z = lane_sum(f.Z);
  if (kEnergy) {
    eb = lane_sum(eb);
    ea = lane_sum(ea);
    ed = lane_sum(ed);
    ex = lane_sum(ex);
    en = lane_sum(en);
  }
  if (q == 0) {
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

// Launch shapes of the force-only kernel the autotuner chooses from: threads per
// block and the minimum resident blocks per SM handed to the register allocator.
// The shape changes neither the per-atom decomposition nor the results.
struct ForceShape {
  int block, min_blocks;
};
static const ForceShape kForceShapes[] = {{128, 1}, {128, 12}, {256, 6}, {64, 24}};

int force_variant_count() { return (int)(sizeof(kForceShapes) / sizeof(kForceShapes[0])); }

void force_variant_shape(int v, int* block, int* min_blocks) {
  *block = kForceShapes[v].block;
  *min_blocks = kForceShapes[v].min_blocks;
}

void launch_force(const Arena& A, int64_t n_atoms_span, bool energy, cudaStream_t st, bool only_rebuilt,
                  int variant) {
  if (n_atoms_span <= 0) return;
  const int ob = only_rebuilt ? 1 : 0;
  if (energy) {
    const int64_t blocks = (n_atoms_span * kLanes + 127) / 128;
    k_force<true, 128, 1><<<(unsigned)blocks, 128, 0, st>>>(A, n_atoms_span, ob);
    return;
  }
  const int bs = kForceShapes[variant].block;
  const unsigned blocks = (unsigned)((n_atoms_span * kLanes + bs - 1) / bs);
  switch (variant) {
    case 1: k_force<false, 128, 12><<<blocks, 128, 0, st>>>(A, n_atoms_span, ob); break;
    case 2: k_force<false, 256, 6><<<blocks, 256, 0, st>>>(A, n_atoms_span, ob); break;
    case 3: k_force<false, 64, 24><<<blocks, 64, 0, st>>>(A, n_atoms_span, ob); break;
    default: k_force<false, 128, 1><<<blocks, 128, 0, st>>>(A, n_atoms_span, ob); break;
  }
}

}  // namespace pq
