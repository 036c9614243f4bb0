// Synthetic poly-alanine-like systems and host-side topology lowering.
//
// The generator stands in for PRISM-PREP output (PrismPrepTopology,
// crates/prism-nhs/src/input.rs:1027-1140): it emits positions, HMR masses,
// charges, per-atom LJ, bonds/angles/dihedrals, exclusions, exact 1-4
// exceptions and hydrogen clusters.  Force-field numbers are the archived
// ff14SB tables (.archive/crates/prism-physics/src/amber_ff14sb.rs:367-741,
// :919-970).  Geometry is grown residue by residue with ideal internal
// coordinates inside a confining sphere or box, rejecting clashes; compact
// systems are grown sparse and then squeezed into their target region
// (squeeze(), below).
//
// All floating-point work here uses IEEE-exact operations and project-written
// series for sin/cos/log, so the same seed yields the same bits on x86-64 and
// on aarch64 (the file is compiled with -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "pq_host.h"

namespace pq {

// --------------------------------------------------------------------------
// Deterministic double-precision helpers.
// --------------------------------------------------------------------------
namespace det {

constexpr double kPi = 3.14159265358979311600;
constexpr double kHalfPi = 1.57079632679489655800;

inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }

// sin/cos of r in [-π/4, π/4] by Taylor series (degree 21/22).
inline void sincos_small(double r, double* s, double* c) {
  const double r2 = r * r;
  double ps = 0.0, pc = 0.0;
  // sin: sum_{k=0}^{10} (-1)^k r^(2k+1)/(2k+1)!  ; cos: sum_{k=0}^{11} (-1)^k r^(2k)/(2k)!
  static const double sc[11] = {1.0,
                                -1.0 / 6.0,
                                1.0 / 120.0,
                                -1.0 / 5040.0,
                                1.0 / 362880.0,
                                -1.0 / 39916800.0,
                                1.0 / 6227020800.0,
                                -1.0 / 1307674368000.0,
                                1.0 / 355687428096000.0,
                                -1.0 / 121645100408832000.0,
                                1.0 / 51090942171709440000.0};
  static const double cc[12] = {1.0,
                                -1.0 / 2.0,
                                1.0 / 24.0,
                                -1.0 / 720.0,
                                1.0 / 40320.0,
                                -1.0 / 3628800.0,
                                1.0 / 479001600.0,
                                -1.0 / 87178291200.0,
                                1.0 / 20922789888000.0,
                                -1.0 / 6402373705728000.0,
                                1.0 / 2432902008176640000.0,
                                -1.0 / 1124000727777607680000.0};
  for (int k = 10; k >= 0; --k) ps = fma_(ps, r2, sc[k]);
  for (int k = 11; k >= 0; --k) pc = fma_(pc, r2, cc[k]);
  *s = r * ps;
  *c = pc;
}

inline void sincos(double x, double* s, double* c) {
  const double q = std::nearbyint(x / kHalfPi);
  const double r = fma_(-q, kHalfPi, x);
  double ss, cc;
  sincos_small(r, &ss, &cc);
  long long qi = (long long)q;
  switch (((qi % 4) + 4) % 4) {
    case 0: *s = ss;  *c = cc;  break;
    case 1: *s = cc;  *c = -ss; break;
    case 2: *s = -ss; *c = -cc; break;
    default: *s = -cc; *c = ss; break;
  }
}

// ln(u), u > 0, via frexp and the atanh series.
inline double log(double u) {
  int e = 0;
  double m = std::frexp(u, &e);  // [0.5, 1)
  if (m < 0.70710678118654752) {
    m = m * 2.0;
    e -= 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 0.0;
  for (int k = 15; k >= 0; --k) p = fma_(p, s2, 1.0 / (double)(2 * k + 1));
  return fma_((double)e, 0.693147180559945286, 2.0 * s * p);
}

// Real cube root by Newton iteration from a fixed start (x > 0).
inline double cbrt(double x) {
  double y = 1.0;
  while (y * y * y < x) y *= 2.0;
  for (int it = 0; it < 200; ++it) {
    const double n = y - (y * y * y - x) / (3.0 * y * y);
    if (n == y) break;
    y = n;
  }
  return y;
}

struct Rng {  // xoshiro256** seeded by splitmix64
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; ++i) {
      z += 0x9E3779B97F4A7C15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double normal() {
    const double u1 = ((double)(next() >> 11) + 1.0) * (1.0 / 9007199254740992.0);  // (0,1]
    const double u2 = uniform();
    double s, c;
    sincos(2.0 * kPi * u2, &s, &c);
    return std::sqrt(-2.0 * det::log(u1)) * c;
  }
};

}  // namespace det

// --------------------------------------------------------------------------
// ff14SB ALA tables (amber_ff14sb.rs).  Atom types used by the residue model.
// --------------------------------------------------------------------------
enum AType : int { T_N = 0, T_H, T_CT, T_H1, T_HC, T_C, T_O };

struct LJType {
  double epsilon, rmin_half;
};
static const LJType kLJ[7] = {
    {0.170, 1.824},   // N
    {0.0157, 0.600},  // H
    {0.1094, 1.908},  // CT
    {0.0157, 1.387},  // H1
    {0.0157, 1.487},  // HC
    {0.0860, 1.908},  // C
    {0.2100, 1.661},  // O
};
static const double kMass[7] = {14.01, 1.008, 12.01, 1.008, 1.008, 12.01, 16.00};

// Residue template: N H CA HA CB HB1 HB2 HB3 C O
static const int kResType[10] = {T_N, T_H, T_CT, T_H1, T_CT, T_HC, T_HC, T_HC, T_C, T_O};
static const double kResCharge[10] = {-0.4157, 0.2719, 0.0337, 0.0823, -0.1825,
                                      0.0603,  0.0603, 0.0603, 0.5973, -0.5679};
enum { A_N = 0, A_H, A_CA, A_HA, A_CB, A_HB1, A_HB2, A_HB3, A_C, A_O };

static bool is_hydrogen(int t) { return t == T_H || t == T_H1 || t == T_HC; }

static bool bond_param(int a, int b, double* r0, double* k) {
  int t1 = std::min(a, b), t2 = std::max(a, b);
  auto is = [&](int x, int y) { return t1 == std::min(x, y) && t2 == std::max(x, y); };
  if (is(T_N, T_H)) { *r0 = 1.010; *k = 434.0; return true; }
  if (is(T_N, T_CT)) { *r0 = 1.449; *k = 337.0; return true; }
  if (is(T_CT, T_C)) { *r0 = 1.522; *k = 317.0; return true; }
  if (is(T_C, T_O)) { *r0 = 1.229; *k = 570.0; return true; }
  if (is(T_N, T_C)) { *r0 = 1.335; *k = 490.0; return true; }
  if (is(T_CT, T_CT)) { *r0 = 1.526; *k = 310.0; return true; }
  if (is(T_CT, T_HC)) { *r0 = 1.090; *k = 340.0; return true; }
  if (is(T_CT, T_H1)) { *r0 = 1.090; *k = 340.0; return true; }
  return false;
}

static bool angle_param(int a, int b, int c, double* th0_deg, double* k) {
  auto m = [&](int x, int y, int z) { return (a == x && b == y && c == z) || (a == z && b == y && c == x); };
  if (m(T_H, T_N, T_CT)) { *th0_deg = 118.0; *k = 50.0; return true; }
  if (m(T_CT, T_N, T_C)) { *th0_deg = 121.9; *k = 50.0; return true; }
  if (m(T_H, T_N, T_C)) { *th0_deg = 119.8; *k = 50.0; return true; }
  if (m(T_N, T_CT, T_C)) { *th0_deg = 110.1; *k = 63.0; return true; }
  if (m(T_N, T_CT, T_CT)) { *th0_deg = 109.7; *k = 80.0; return true; }
  if (m(T_CT, T_CT, T_C)) { *th0_deg = 111.1; *k = 63.0; return true; }
  if (m(T_CT, T_C, T_O)) { *th0_deg = 120.4; *k = 80.0; return true; }
  if (m(T_CT, T_C, T_N)) { *th0_deg = 116.6; *k = 70.0; return true; }
  if (m(T_O, T_C, T_N)) { *th0_deg = 122.9; *k = 80.0; return true; }
  if (m(T_N, T_CT, T_H1)) { *th0_deg = 109.5; *k = 50.0; return true; }
  if (m(T_C, T_CT, T_H1)) { *th0_deg = 109.5; *k = 50.0; return true; }
  if (m(T_H1, T_CT, T_CT)) { *th0_deg = 109.5; *k = 50.0; return true; }
  if (m(T_CT, T_CT, T_HC)) { *th0_deg = 109.5; *k = 50.0; return true; }
  if (m(T_HC, T_CT, T_HC)) { *th0_deg = 109.5; *k = 35.0; return true; }
  return false;
}

struct TorsionTerm {
  double k;
  int n;
  double phase_deg;
};

// Specific matches first, then the generic central-bond entries.  Terms with
// a zero barrier are not emitted.
static std::vector<TorsionTerm> torsion_params(int a, int b, int c, int d) {
  auto spec = [&](int w, int x, int y, int z) {
    return (a == w && b == x && c == y && d == z) || (a == z && b == y && c == x && d == w);
  };
  if (spec(T_C, T_N, T_CT, T_C)) return {};                              // φ: k = 0
  if (spec(T_N, T_CT, T_C, T_N)) return {{0.4, 1, 0.0}, {2.0, 2, 180.0}};  // ψ
  if (spec(T_CT, T_C, T_N, T_CT)) return {{2.5, 2, 180.0}};               // ω
  auto cen = [&](int x, int y) { return (b == x && c == y) || (b == y && c == x); };
  if (cen(T_C, T_N)) return {{2.5, 2, 180.0}};
  if (cen(T_CT, T_CT)) return {{0.156, 3, 0.0}};
  return {};  // X-C-CT-X and X-CT-N-X carry k = 0
}

// --------------------------------------------------------------------------
// Geometry helpers.
// --------------------------------------------------------------------------
struct V3 {
  double x, y, z;
};
static V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static V3 unit(V3 a) {
  const double n = std::sqrt(dot(a, a));
  return (1.0 / n) * a;
}

// Place D with |CD| = r, angle BCD = theta, dihedral ABCD = phi (radians).
static V3 place(V3 A, V3 B, V3 C, double r, double theta, double phi) {
  const V3 bc = unit(C - B);
  const V3 n = unit(cross(B - A, bc));
  const V3 m = cross(n, bc);
  double st, ct, sp, cp;
  det::sincos(theta, &st, &ct);
  det::sincos(phi, &sp, &cp);
  const double dx = -r * ct, dy = r * st * cp, dz = r * st * sp;
  return C + dx * bc + dy * m + dz * n;
}

static double deg(double d) { return d * (det::kPi / 180.0); }

struct Region {
  bool sphere;
  V3 center;
  double radius;
  V3 lo, hi;
  // Optional pull point of the growth (a chain's slot inside a shared box):
  // the first residue starts near it and candidates are weighted toward it.
  bool has_pull = false;
  V3 pull;
  double pull_scale = 0.0;
  bool inside(V3 p, double margin) const {
    if (sphere) {
      const V3 d = p - center;
      const double r = radius - margin;
      return dot(d, d) <= r * r;
    }
    return p.x >= lo.x + margin && p.x <= hi.x - margin && p.y >= lo.y + margin &&
           p.y <= hi.y - margin && p.z >= lo.z + margin && p.z <= hi.z - margin;
  }
};

// Spatial hash of placed atoms for clash checks (LIFO removal on backtrack).
struct ClashGrid {
  double cell = 3.2;
  std::unordered_map<int64_t, std::vector<int>> cells;
  static int64_t key(long long ix, long long iy, long long iz) {
    return ((ix + 1048576) << 42) | ((iy + 1048576) << 21) | (iz + 1048576);
  }
  void coords(V3 p, long long* ix, long long* iy, long long* iz) const {
    *ix = (long long)std::floor(p.x / cell);
    *iy = (long long)std::floor(p.y / cell);
    *iz = (long long)std::floor(p.z / cell);
  }
  void add(int id, V3 p) {
    long long ix, iy, iz;
    coords(p, &ix, &iy, &iz);
    cells[key(ix, iy, iz)].push_back(id);
  }
  void remove(int id, V3 p) {
    long long ix, iy, iz;
    coords(p, &ix, &iy, &iz);
    auto& v = cells[key(ix, iy, iz)];
    if (!v.empty() && v.back() == id) v.pop_back();
    else v.erase(std::remove(v.begin(), v.end(), id), v.end());
  }
};

struct Builder {
  std::vector<V3> pos;
  std::vector<int> type;
  std::vector<int> chain_of;
  std::vector<int> res_of;  // global residue index
  ClashGrid grid;

  static double min_dist(int ta, int tb) {
    const bool ha = is_hydrogen(ta), hb = is_hydrogen(tb);
    if (ha && hb) return 1.8;
    if (ha || hb) return 1.9;
    return 2.8;
  }
};

// Geometry of one residue given the previous residue's backbone.
struct ResGeom {
  V3 a[10];
};

static ResGeom build_residue(const ResGeom* prev, double prev_psi, double phi, double psi,
                             V3 n0, V3 ca_dir, V3 up) {
  ResGeom g;
  if (!prev) {
    g.a[A_N] = n0;
    g.a[A_CA] = n0 + 1.449 * ca_dir;
    // C from a virtual frame point
    const V3 virt = n0 + up;
    g.a[A_C] = place(virt, g.a[A_N], g.a[A_CA], 1.522, deg(110.1), phi);
    g.a[A_H] = place(g.a[A_C], g.a[A_CA], g.a[A_N], 1.010, deg(118.0), deg(180.0));
  } else {
    g.a[A_N] = place(prev->a[A_N], prev->a[A_CA], prev->a[A_C], 1.335, deg(116.6), prev_psi);
    g.a[A_CA] = place(prev->a[A_CA], prev->a[A_C], g.a[A_N], 1.449, deg(121.9), deg(180.0));
    g.a[A_C] = place(prev->a[A_C], g.a[A_N], g.a[A_CA], 1.522, deg(110.1), phi);
    g.a[A_H] = place(prev->a[A_O], prev->a[A_C], g.a[A_N], 1.010, deg(119.8), deg(180.0));
  }
  g.a[A_O] = place(g.a[A_N], g.a[A_CA], g.a[A_C], 1.229, deg(120.4), psi + deg(180.0));
  g.a[A_CB] = place(g.a[A_C], g.a[A_N], g.a[A_CA], 1.526, deg(109.7), deg(-122.5));
  g.a[A_HA] = place(g.a[A_C], g.a[A_N], g.a[A_CA], 1.090, deg(109.5), deg(117.0));
  g.a[A_HB1] = place(g.a[A_N], g.a[A_CA], g.a[A_CB], 1.090, deg(109.5), deg(60.0));
  g.a[A_HB2] = place(g.a[A_N], g.a[A_CA], g.a[A_CB], 1.090, deg(109.5), deg(180.0));
  g.a[A_HB3] = place(g.a[A_N], g.a[A_CA], g.a[A_CB], 1.090, deg(109.5), deg(-60.0));
  return g;
}

static void sample_phipsi(det::Rng& rng, double* phi, double* psi) {
  const double u = rng.uniform();
  double p0, s0;
  if (u < 0.45) { p0 = -63.0; s0 = -42.0; }
  else if (u < 0.80) { p0 = -120.0; s0 = 130.0; }
  else if (u < 0.95) { p0 = -70.0; s0 = 145.0; }
  else { p0 = 60.0; s0 = 45.0; }
  *phi = deg(p0 + 12.0 * rng.normal());
  *psi = deg(s0 + 12.0 * rng.normal());
}

// Atoms of the previous residue that are within three bonds of the new one
// and therefore skipped by the clash test.
static bool skip_prev(int slot) {
  return slot == A_N || slot == A_CA || slot == A_C || slot == A_O || slot == A_HA || slot == A_CB ||
         slot == A_H;
}

// True when residue geometry g (index r of the chain) is inside the region and
// clears every placed atom except the covalent neighbourhood in residue r-1.
static bool residue_fits(const Builder& B, const ResGeom& g, int chain, int r, int res_base,
                         size_t atom_base, const Region& reg) {
  for (int s = 0; s < 10; ++s)
    if (!reg.inside(g.a[s], 1.5)) return false;
  for (int s = 0; s < 10; ++s) {
    const V3 p = g.a[s];
    long long ix, iy, iz;
    B.grid.coords(p, &ix, &iy, &iz);
    for (long long dz = -1; dz <= 1; ++dz)
      for (long long dy = -1; dy <= 1; ++dy)
        for (long long dx = -1; dx <= 1; ++dx) {
          auto it = B.grid.cells.find(ClashGrid::key(ix + dx, iy + dy, iz + dz));
          if (it == B.grid.cells.end()) continue;
          for (int other : it->second) {
            if (B.chain_of[other] == chain && B.res_of[other] == res_base + r - 1 &&
                skip_prev((int)((other - atom_base) % 10)))
              continue;
            const V3 d = B.pos[other] - p;
            const double md = Builder::min_dist(kResType[s], B.type[other]);
            if (dot(d, d) < md * md) return false;
          }
        }
  }
  return true;
}

// Configurational-bias growth: each residue draws K (φ, ψ) candidates, keeps
// those that fit, and picks one with weight exp(-3 (|CA - centre| / R)^2) so
// the chain folds back into its region; dead ends back up by a depth that
// grows with repeated failure.
static bool grow_chain(Builder& B, int chain, int n_res, int res_base, const Region& reg, det::Rng& rng) {
  const size_t atom_base = B.pos.size();
  std::vector<ResGeom> geo;
  std::vector<double> psis;
  geo.reserve(n_res);
  const int K = 16;
  V3 centre = reg.center;
  double scale = reg.radius;
  if (!reg.sphere) {
    centre = 0.5 * (reg.lo + reg.hi);
    const V3 h = 0.5 * (reg.hi - reg.lo);
    scale = std::max(h.x, std::max(h.y, h.z));
  }
  if (reg.has_pull) {
    centre = reg.pull;
    scale = reg.pull_scale;
  }
  long long attempts = 0;
  const long long max_attempts = 400LL * n_res + 2000;
  int fails = 0;
  while ((int)geo.size() < n_res) {
    if (++attempts > max_attempts) return false;
    const int r = (int)geo.size();
    ResGeom cand[K];
    double psi_c[K], w[K];
    int nvalid = 0;
    double wsum = 0.0;
    for (int k = 0; k < K; ++k) {
      double phi, psi;
      sample_phipsi(rng, &phi, &psi);
      ResGeom g;
      if (r == 0) {
        V3 start = centre;
        for (int t = 0; t < 1000; ++t) {
          const V3 off{(rng.uniform() * 2 - 1) * scale * 0.5, (rng.uniform() * 2 - 1) * scale * 0.5,
                       (rng.uniform() * 2 - 1) * scale * 0.5};
          start = centre + off;
          if (reg.inside(start, 4.0)) break;
        }
        const V3 dir = unit(V3{rng.normal(), rng.normal(), rng.normal()});
        const V3 up = unit(cross(dir, V3{0.3, 0.5, 0.8}));
        g = build_residue(nullptr, 0.0, phi, psi, start, dir, up);
      } else {
        g = build_residue(&geo[r - 1], psis[r - 1], phi, psi, V3{}, V3{}, V3{});
      }
      if (!residue_fits(B, g, chain, r, res_base, atom_base, reg)) continue;
      const V3 d = g.a[A_CA] - centre;
      const double q = std::sqrt(dot(d, d)) / scale;
      cand[nvalid] = g;
      psi_c[nvalid] = psi;
      w[nvalid] = std::exp(-3.0 * q * q);
      wsum += w[nvalid];
      ++nvalid;
    }
    if (nvalid == 0) {
      ++fails;
      const int depth = std::min<int>((int)geo.size(), 1 + (int)(rng.uniform() * std::min(2 + fails / 4, 24)));
      for (int k = 0; k < depth; ++k) {
        const int rr = (int)geo.size() - 1;
        for (int s = 9; s >= 0; --s) {
          const int id = (int)(atom_base + (size_t)rr * 10 + (size_t)s);
          B.grid.remove(id, B.pos[id]);
        }
        B.pos.resize(B.pos.size() - 10);
        B.type.resize(B.type.size() - 10);
        B.chain_of.resize(B.chain_of.size() - 10);
        B.res_of.resize(B.res_of.size() - 10);
        geo.pop_back();
        psis.pop_back();
      }
      continue;
    }
    if (fails > 0) --fails;
    double u = rng.uniform() * wsum;
    int pick = nvalid - 1;
    for (int k = 0; k < nvalid; ++k) {
      u -= w[k];
      if (u <= 0.0) {
        pick = k;
        break;
      }
    }
    const ResGeom& g = cand[pick];
    for (int s = 0; s < 10; ++s) {
      const int id = (int)B.pos.size();
      B.pos.push_back(g.a[s]);
      B.type.push_back(kResType[s]);
      B.chain_of.push_back(chain);
      B.res_of.push_back(res_base + r);
      B.grid.add(id, g.a[s]);
    }
    geo.push_back(g);
    psis.push_back(psi_c[pick]);
  }
  return true;
}

// Choose gx*gy*gz == n with the smallest aspect ratio (falls back to a cube).
static void split_box(int n, int* gx, int* gy, int* gz) {
  double best = 1e30;
  *gx = *gy = *gz = 1;
  for (int a = 1; a <= n; ++a)
    for (int b = a; a * b <= n; ++b) {
      if (n % (a * b)) continue;
      const int c = n / (a * b);
      if (c < b) continue;
      const double ratio = (double)c / (double)a;
      if (ratio < best) {
        best = ratio;
        *gx = a;
        *gy = b;
        *gz = c;
      }
    }
  if (best > 4.0) {
    int k = 1;
    while (k * k * k < n) ++k;
    *gx = *gy = *gz = k;
  }
}

// --------------------------------------------------------------------------
// Topology assembly (bonded terms, exclusions, exceptions, clusters, HMR).
// --------------------------------------------------------------------------
static void assemble(const Builder& B, int n_chains, int n_res, HostTopology* T) {
  const int n = (int)B.pos.size();
  T->n_atoms = n;
  T->positions.resize(3 * (size_t)n);
  T->masses.resize(n);
  T->charges.resize(n);
  T->lj_sigma.resize(n);
  T->lj_epsilon.resize(n);
  std::vector<double> mass(n);
  for (int a = 0; a < n; ++a) {
    T->positions[3 * a + 0] = (float)B.pos[a].x;
    T->positions[3 * a + 1] = (float)B.pos[a].y;
    T->positions[3 * a + 2] = (float)B.pos[a].z;
    const int t = B.type[a];
    const int slot = a % 10;
    T->charges[a] = (float)kResCharge[slot];
    // sigma = 2 * rmin/2 * 2^(-1/6)
    T->lj_sigma[a] = (float)(2.0 * kLJ[t].rmin_half * 0.89089871814033930);
    T->lj_epsilon[a] = (float)kLJ[t].epsilon;
    mass[a] = kMass[t];
  }
  // bond graph
  std::vector<std::vector<int>> adj(n);
  auto add_bond = [&](int i, int j) {
    double r0, k;
    bond_param(B.type[i], B.type[j], &r0, &k);
    T->bonds.push_back({i, j, (float)r0, (float)k});
    adj[i].push_back(j);
    adj[j].push_back(i);
  };
  for (int c = 0; c < n_chains; ++c) {
    for (int r = 0; r < n_res; ++r) {
      const int b = (c * n_res + r) * 10;
      add_bond(b + A_N, b + A_H);
      add_bond(b + A_N, b + A_CA);
      add_bond(b + A_CA, b + A_HA);
      add_bond(b + A_CA, b + A_CB);
      add_bond(b + A_CB, b + A_HB1);
      add_bond(b + A_CB, b + A_HB2);
      add_bond(b + A_CB, b + A_HB3);
      add_bond(b + A_CA, b + A_C);
      add_bond(b + A_C, b + A_O);
      if (r + 1 < n_res) add_bond(b + A_C, b + 10 + A_N);
    }
  }
  for (auto& v : adj) std::sort(v.begin(), v.end());
  // angles: j central, i < k
  for (int j = 0; j < n; ++j) {
    for (size_t x = 0; x < adj[j].size(); ++x)
      for (size_t y = x + 1; y < adj[j].size(); ++y) {
        const int i = adj[j][x], k = adj[j][y];
        double th, kk;
        if (angle_param(B.type[i], B.type[j], B.type[k], &th, &kk))
          T->angles.push_back({i, j, k, (float)deg(th), (float)kk});
      }
  }
  // proper torsions over each bond j-k (j < k), i ∈ adj(j)\{k}, l ∈ adj(k)\{j}
  for (int j = 0; j < n; ++j)
    for (int k : adj[j]) {
      if (k <= j) continue;
      for (int i : adj[j]) {
        if (i == k) continue;
        for (int l : adj[k]) {
          if (l == j || l == i) continue;
          for (const TorsionTerm& t : torsion_params(B.type[i], B.type[j], B.type[k], B.type[l]))
            T->dihedrals.push_back({i, j, k, l, t.n, (float)deg(t.phase_deg), (float)t.k});
        }
      }
    }
  // topological distance ≤ 3 → exclusions; exactly 3 → exceptions
  std::vector<std::vector<int>> excl(n);
  for (int a = 0; a < n; ++a) {
    std::vector<int> d1 = adj[a], d2, d3;
    for (int b : d1)
      for (int c2 : adj[b])
        if (c2 != a) d2.push_back(c2);
    for (int b : d2)
      for (int c3 : adj[b])
        if (c3 != a) d3.push_back(c3);
    std::vector<int> all;
    all.insert(all.end(), d1.begin(), d1.end());
    all.insert(all.end(), d2.begin(), d2.end());
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    std::vector<int> third;
    for (int x : d3)
      if (!std::binary_search(all.begin(), all.end(), x) && x != a) third.push_back(x);
    std::sort(third.begin(), third.end());
    third.erase(std::unique(third.begin(), third.end()), third.end());
    for (int x : third) {
      if (a < x) {
        const double qq = kResCharge[a % 10] * kResCharge[x % 10] / 1.2;
        const double sig = 0.5 * ((double)T->lj_sigma[a] + (double)T->lj_sigma[x]);
        const double eps = 0.5 * std::sqrt((double)T->lj_epsilon[a] * (double)T->lj_epsilon[x]);
        T->exceptions.push_back({a, x, (float)qq, (float)sig, (float)eps});
      }
    }
    all.insert(all.end(), third.begin(), third.end());
    std::sort(all.begin(), all.end());
    excl[a] = all;
  }
  T->exclusion_offsets.assign(1, 0);
  for (int a = 0; a < n; ++a) {
    T->exclusions.insert(T->exclusions.end(), excl[a].begin(), excl[a].end());
    T->exclusion_offsets.push_back((int32_t)T->exclusions.size());
  }
  // hydrogen clusters (NH, CH, CH3) and HMR ×3 (input.rs:2482-2560)
  const double factor = 3.0;
  for (int c = 0; c < n_chains; ++c)
    for (int r = 0; r < n_res; ++r) {
      const int b = (c * n_res + r) * 10;
      const int centers[3] = {b + A_N, b + A_CA, b + A_CB};
      for (int ci = 0; ci < 3; ++ci) {
        const int cen = centers[ci];
        prismq_hcluster hc;
        std::memset(&hc, 0, sizeof(hc));
        hc.central_atom = cen;
        hc.hydrogen_atoms[0] = hc.hydrogen_atoms[1] = hc.hydrogen_atoms[2] = -1;
        int nh = 0;
        for (int nb : adj[cen])
          if (is_hydrogen(B.type[nb])) {
            hc.hydrogen_atoms[nh] = nb;
            hc.bond_lengths[nh] = (float)(B.type[nb] == T_H ? 1.010 : 1.090);
            ++nh;
          }
        hc.n_hydrogens = nh;
        const double m_h = kMass[T_H] * factor;
        const double m_c = mass[cen] - nh * (m_h - kMass[T_H]);
        mass[cen] = m_c;
        for (int h = 0; h < nh; ++h) mass[hc.hydrogen_atoms[h]] = m_h;
        hc.inv_mass_central = (float)(1.0 / m_c);
        hc.inv_mass_h = (float)(1.0 / m_h);
        T->clusters.push_back(hc);
      }
    }
  for (int a = 0; a < n; ++a) T->masses[a] = (float)mass[a];
}

// --------------------------------------------------------------------------
// Compaction: the grown chains are squeezed into their target region by a
// FIRE relaxation (Bitzek et al., Phys. Rev. Lett. 97, 170201 (2006)) of a
// restraint energy while a wall shrinks from the grown extent to the target:
//   bonds   k_b (r - r0)^2                 (r0 from the topology)
//   angles  k_a (cos θ - cos θ0)^2         (θ0 from the topology)
//   contact k_r (d_ij - r)^2 for r < d_ij  (every pair more than three bonds
//           apart; d_ij = max(0.8 (Rmin_i/2 + Rmin_j/2), 2 Å) from the ff14SB
//           LJ radii)
//   wall    k_w s^2, s the distance of an atom outside the region.
// Arithmetic is +, -, *, / and sqrt in a fixed order (sums over atoms run in
// index order), so the result has the same bits on every IEEE machine.  After
// the relaxation each hydrogen is moved along its bond to the constraint
// length, so SHAKE starts from satisfied constraints.
// --------------------------------------------------------------------------
struct SqueezeRegion {
  bool sphere = true;
  std::vector<V3> centre;  // per chain (sphere systems)
  double r_start = 0.0, r_target = 0.0;
  V3 lo0, hi0, lo1, hi1;  // box: start and target
};

struct SqueezeReport {
  int iterations = 0;
  double max_overlap = 0.0;   // max (d_ij - r) over contact pairs
  double max_outside = 0.0;   // max wall violation (Å)
  double min_nonbonded = 0.0; // closest pair more than three bonds apart (Å)
};

static double contact_radius(int type) { return kLJ[type].rmin_half; }

static void squeeze(HostTopology* T, const std::vector<int>& types, int atoms_per_chain, const SqueezeRegion& reg,
                    SqueezeReport* rep) {
  const int n = T->n_atoms;
  const size_t n3 = 3 * (size_t)n;
  std::vector<double> x(n3), v(n3, 0.0), f(n3), xl(n3);
  for (size_t k = 0; k < n3; ++k) x[k] = (double)T->positions[k];
  const double kb = 100.0, ka = 50.0, kr = 50.0, kw = 100.0;
  std::vector<double> cos0(T->angles.size());
  for (size_t t = 0; t < T->angles.size(); ++t) {
    double s, c;
    det::sincos((double)T->angles[t].theta0, &s, &c);
    cos0[t] = c;
  }
  std::vector<double> rad(n);
  double rad_max = 0.0;
  for (int a = 0; a < n; ++a) {
    rad[a] = contact_radius(types[a]);
    rad_max = std::max(rad_max, rad[a]);
  }
  const double dmax = std::max(2.0, 1.6 * rad_max);
  const double skin = 1.2, rl = dmax + skin, rl2 = rl * rl;
  const int32_t* eo = T->exclusion_offsets.data();
  const int32_t* ex = T->exclusions.data();
  auto excluded = [&](int i, int j) { return std::binary_search(ex + eo[i], ex + eo[i + 1], j); };
  // Contact pairs within rl (i < j) in the order of i, then of the cell walk
  // (cells hold atoms in index order), which is fixed by the positions.
  std::vector<int> pi_, pj_;
  std::vector<double> pd;
  std::vector<int> head, order, cell;
  double shrink_since_build = 1.0;  // product of the scale factors applied since the last build
  auto build_pairs = [&]() {
    pi_.clear();
    pj_.clear();
    pd.clear();
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < n; ++a)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], x[3 * a + d]);
        hi[d] = std::max(hi[d], x[3 * a + d]);
      }
    long long dims[3];
    double inv[3];
    for (int d = 0; d < 3; ++d) {
      dims[d] = std::max(1LL, (long long)((hi[d] - lo[d]) / rl));
      inv[d] = (double)dims[d] / (hi[d] - lo[d] + 1e-9);
    }
    const long long ncell = dims[0] * dims[1] * dims[2];
    head.assign(ncell + 1, 0);
    order.resize(n);
    cell.resize(n);
    for (int a = 0; a < n; ++a) {
      long long c3[3];
      for (int d = 0; d < 3; ++d) {
        const long long c = (long long)((x[3 * a + d] - lo[d]) * inv[d]);
        c3[d] = std::min(std::max(c, 0LL), dims[d] - 1);
      }
      cell[a] = (int)(c3[0] + dims[0] * (c3[1] + dims[1] * c3[2]));
      head[cell[a] + 1] += 1;
    }
    for (long long c = 0; c < ncell; ++c) head[c + 1] += head[c];
    {
      std::vector<int> cur(head.begin(), head.end() - 1);
      for (int a = 0; a < n; ++a) order[cur[cell[a]]++] = a;
    }
    for (int a = 0; a < n; ++a) {
      const long long c = cell[a];
      const long long cx = c % dims[0], cy = (c / dims[0]) % dims[1], cz = c / (dims[0] * dims[1]);
      const double xa = x[3 * a], ya = x[3 * a + 1], za = x[3 * a + 2];
      for (long long dz = -1; dz <= 1; ++dz)
        for (long long dy = -1; dy <= 1; ++dy)
          for (long long dx = -1; dx <= 1; ++dx) {
            const long long X = cx + dx, Y = cy + dy, Z = cz + dz;
            if (X < 0 || Y < 0 || Z < 0 || X >= dims[0] || Y >= dims[1] || Z >= dims[2]) continue;
            const long long o = X + dims[0] * (Y + dims[1] * Z);
            for (int k = head[o]; k < head[o + 1]; ++k) {
              const int b = order[k];
              if (b <= a) continue;
              const double ddx = x[3 * b] - xa, ddy = x[3 * b + 1] - ya, ddz = x[3 * b + 2] - za;
              if (ddx * ddx + ddy * ddy + ddz * ddz > rl2) continue;
              if (excluded(a, b)) continue;
              pi_.push_back(a);
              pj_.push_back(b);
              pd.push_back(std::max(0.8 * (rad[a] + rad[b]), 2.0));
            }
          }
    }
    xl = x;
    shrink_since_build = 1.0;
  };
  double max_overlap = 0.0, max_outside = 0.0;
  auto forces = [&](bool wall) {
    std::fill(f.begin(), f.end(), 0.0);
    for (const prismq_bond& b : T->bonds) {
      const int i = b.i, j = b.j;
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (r < 1e-9) continue;
      const double s = 2.0 * kb * (r - (double)b.r0) / r;  // pulls i toward j when stretched
      f[3 * i] += s * dx; f[3 * i + 1] += s * dy; f[3 * i + 2] += s * dz;
      f[3 * j] -= s * dx; f[3 * j + 1] -= s * dy; f[3 * j + 2] -= s * dz;
    }
    for (size_t t = 0; t < T->angles.size(); ++t) {
      const prismq_angle& g = T->angles[t];
      const int i = g.i, j = g.j, k = g.k;
      const double ux = x[3 * i] - x[3 * j], uy = x[3 * i + 1] - x[3 * j + 1], uz = x[3 * i + 2] - x[3 * j + 2];
      const double wx = x[3 * k] - x[3 * j], wy = x[3 * k + 1] - x[3 * j + 1], wz = x[3 * k + 2] - x[3 * j + 2];
      const double uu = ux * ux + uy * uy + uz * uz, ww = wx * wx + wy * wy + wz * wz;
      if (uu < 1e-18 || ww < 1e-18) continue;
      const double inv = 1.0 / (std::sqrt(uu) * std::sqrt(ww));
      const double c = (ux * wx + uy * wy + uz * wz) * inv;
      const double g2 = -2.0 * ka * (c - cos0[t]);  // -dE/dc
      const double ai = c / uu, ak = c / ww;
      const double fix = g2 * (wx * inv - ai * ux), fiy = g2 * (wy * inv - ai * uy), fiz = g2 * (wz * inv - ai * uz);
      const double fkx = g2 * (ux * inv - ak * wx), fky = g2 * (uy * inv - ak * wy), fkz = g2 * (uz * inv - ak * wz);
      f[3 * i] += fix; f[3 * i + 1] += fiy; f[3 * i + 2] += fiz;
      f[3 * k] += fkx; f[3 * k + 1] += fky; f[3 * k + 2] += fkz;
      f[3 * j] -= fix + fkx; f[3 * j + 1] -= fiy + fky; f[3 * j + 2] -= fiz + fkz;
    }
    max_overlap = 0.0;
    for (size_t p = 0; p < pi_.size(); ++p) {
      const int i = pi_[p], j = pj_[p];
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
      const double r2 = dx * dx + dy * dy + dz * dz, d = pd[p];
      if (r2 >= d * d) continue;
      const double r = std::sqrt(r2);
      if (r < 1e-9) continue;
      max_overlap = std::max(max_overlap, d - r);
      const double s = 2.0 * kr * (d - r) / r;  // pushes i away from j
      f[3 * i] -= s * dx; f[3 * i + 1] -= s * dy; f[3 * i + 2] -= s * dz;
      f[3 * j] += s * dx; f[3 * j + 1] += s * dy; f[3 * j + 2] += s * dz;
    }
    max_outside = 0.0;
    if (!wall) return;
    if (reg.sphere) {
      const double R = reg.r_target;
      for (int a = 0; a < n; ++a) {
        const V3 c = reg.centre[a / atoms_per_chain];
        const double dx = x[3 * a] - c.x, dy = x[3 * a + 1] - c.y, dz = x[3 * a + 2] - c.z;
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (r <= R) continue;
        const double s = r - R;
        max_outside = std::max(max_outside, s);
        const double g = -2.0 * kw * s / r;
        f[3 * a] += g * dx; f[3 * a + 1] += g * dy; f[3 * a + 2] += g * dz;
      }
    } else {
      const double lo[3] = {reg.lo1.x, reg.lo1.y, reg.lo1.z}, hi[3] = {reg.hi1.x, reg.hi1.y, reg.hi1.z};
      for (int a = 0; a < n; ++a)
        for (int d = 0; d < 3; ++d) {
          const double p = x[3 * a + d];
          if (p > hi[d]) {
            max_outside = std::max(max_outside, p - hi[d]);
            f[3 * a + d] -= 2.0 * kw * (p - hi[d]);
          } else if (p < lo[d]) {
            max_outside = std::max(max_outside, lo[d] - p);
            f[3 * a + d] += 2.0 * kw * (lo[d] - p);
          }
        }
    }
  };
  // One compression step: every atom moves toward its region's centre by the
  // factor s (the list-build positions too, so the displacement test below
  // sees only the relaxation's own motion).
  auto scale_all = [&](double s) {
    for (int a = 0; a < n; ++a) {
      V3 c;
      if (reg.sphere) {
        c = reg.centre[a / atoms_per_chain];
      } else {
        c = 0.5 * (reg.lo0 + reg.hi0);
      }
      const double cc[3] = {c.x, c.y, c.z};
      for (int d = 0; d < 3; ++d) {
        x[3 * a + d] = cc[d] + s * (x[3 * a + d] - cc[d]);
        xl[3 * a + d] = cc[d] + s * (xl[3 * a + d] - cc[d]);
      }
    }
    shrink_since_build *= s;
  };
  // FIRE parameters (Bitzek et al. 2006), unit masses
  const double dt_max = 0.08, f_inc = 1.1, f_dec = 0.5, a_start = 0.1, f_a = 0.99, max_step = 0.1;
  const int n_min = 5;
  double dt = 0.02, alpha = a_start;
  int n_pos = 0;
  auto fire_step = [&](bool wall) {
    forces(wall);
    double P = 0.0, vv = 0.0, ff = 0.0;
    for (size_t k = 0; k < n3; ++k) {
      P += f[k] * v[k];
      vv += v[k] * v[k];
      ff += f[k] * f[k];
    }
    if (P > 0.0) {
      const double sc = ff > 0.0 ? alpha * std::sqrt(vv) / std::sqrt(ff) : 0.0;
      for (size_t k = 0; k < n3; ++k) v[k] = (1.0 - alpha) * v[k] + sc * f[k];
      if (n_pos > n_min) {
        dt = std::min(dt * f_inc, dt_max);
        alpha *= f_a;
      }
      ++n_pos;
    } else {
      std::fill(v.begin(), v.end(), 0.0);
      dt *= f_dec;
      alpha = a_start;
      n_pos = 0;
    }
    double moved2 = 0.0;
    for (int a = 0; a < n; ++a) {
      double* va = &v[3 * (size_t)a];
      const double* fa = &f[3 * (size_t)a];
      for (int d = 0; d < 3; ++d) va[d] += fa[d] * dt;
      const double sp = std::sqrt(va[0] * va[0] + va[1] * va[1] + va[2] * va[2]) * dt;
      const double cap = sp > max_step ? max_step / sp : 1.0;
      for (int d = 0; d < 3; ++d) {
        va[d] *= cap;
        x[3 * (size_t)a + d] += va[d] * dt;
      }
      const double ddx = x[3 * a] - xl[3 * a], ddy = x[3 * a + 1] - xl[3 * a + 1], ddz = x[3 * a + 2] - xl[3 * a + 2];
      moved2 = std::max(moved2, ddx * ddx + ddy * ddy + ddz * ddz);
    }
    // A pair farther than rl at the build is farther than
    // shrink·rl - 2·moved now, which must stay above the largest contact distance.
    if (rl * shrink_since_build - 2.0 * std::sqrt(moved2) < dmax) build_pairs();
  };
  // compression: shrink_steps scale steps of equal ratio, relaxing in between
  double total = 1.0;
  if (reg.sphere) {
    total = reg.r_target / reg.r_start;
  } else {
    total = (reg.hi1.x - reg.lo1.x) / (reg.hi0.x - reg.lo0.x);
  }
  const int shrink_steps = 160, relax_per_step = 3, max_final = 2000;
  int it = 0;
  build_pairs();
  // the per-step ratio total^(1/shrink_steps) by bisection (only IEEE operations)
  double ratio = 1.0;
  if (total < 1.0) {
    double lo_r = total, hi_r = 1.0;
    for (int k = 0; k < 200; ++k) {
      const double mid = 0.5 * (lo_r + hi_r);
      double p = 1.0;
      for (int q = 0; q < shrink_steps; ++q) p *= mid;
      if (p < total) lo_r = mid; else hi_r = mid;
    }
    ratio = hi_r;
    for (int k = 0; k < shrink_steps; ++k) {
      scale_all(ratio);
      for (int r = 0; r < relax_per_step; ++r, ++it) fire_step(false);
    }
  }
  for (int k = 0; k < max_final; ++k, ++it) {
    fire_step(true);
    if (max_overlap < 0.1 && max_outside < 0.1) break;
  }
  // hydrogens onto their constraint lengths
  for (const prismq_hcluster& c : T->clusters) {
    const int ca = c.central_atom;
    for (int h = 0; h < c.n_hydrogens; ++h) {
      const int ha = c.hydrogen_atoms[h];
      const double dx = x[3 * ha] - x[3 * ca], dy = x[3 * ha + 1] - x[3 * ca + 1], dz = x[3 * ha + 2] - x[3 * ca + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (r < 1e-9) continue;
      const double s = (double)c.bond_lengths[h] / r;
      x[3 * ha] = x[3 * ca] + dx * s;
      x[3 * ha + 1] = x[3 * ca + 1] + dy * s;
      x[3 * ha + 2] = x[3 * ca + 2] + dz * s;
    }
  }
  for (size_t k = 0; k < x.size(); ++k) T->positions[k] = (float)x[k];
  if (rep) {
    rep->iterations = it;
    rep->max_overlap = max_overlap;
    rep->max_outside = max_outside;
    build_pairs();
    double mn = 1e300;
    for (size_t p = 0; p < pi_.size(); ++p) {
      const int i = pi_[p], j = pj_[p];
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
      mn = std::min(mn, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    rep->min_nonbonded = pi_.empty() ? 0.0 : mn;
  }
}

// Default target density of the compacted systems: 2,500 atoms in a 40 Å
// globule (a sphere of radius 20 Å).
constexpr double kGlobuleDensity = 2500.0 / (4.0 / 3.0 * det::kPi * 8000.0);
// Density at which the chains are grown before they are squeezed.
constexpr double kGrowDensity = 0.02;

bool polyala_build(int n_chains, int n_res, uint64_t seed, double density, double box_edge,
                   HostTopology* T, std::string* err, int compact, double* squeeze_stats) {
  if (n_chains < 1 || n_res < 1 || n_chains > 100000 || (long long)n_chains * n_res * 10 > 50000000LL) {
    *err = "polyala_build: n_chains/n_residues out of range";
    return false;
  }
  if (!(density > 0.0)) density = compact ? kGlobuleDensity : kGrowDensity;
  const int atoms_per_chain = n_res * 10;
  const double n_total = (double)n_chains * atoms_per_chain;
  // Compacted systems grow at kGrowDensity in an enlarged region first.
  double grow_density = density, grow_box = box_edge;
  if (compact) {
    grow_density = std::min(density, kGrowDensity);
    if (box_edge > 0.0) grow_box = std::max(box_edge, det::cbrt(n_total / kGrowDensity));
  }
  // A region that is too dense for self-avoiding growth is enlarged by 5% in
  // radius (or edge) per attempt.
  for (int attempt = 0; attempt < 16; ++attempt) {
    Builder B;
    det::Rng rng(seed * 0x9E3779B97F4A7C15ull + 0x5052495351ull + (uint64_t)attempt);
    const double grow = 1.0 + 0.05 * attempt;
    bool ok = true;
    int gx = 1, gy = 1, gz = 1;
    if (grow_box > 0.0) split_box(n_chains, &gx, &gy, &gz);
    SqueezeRegion sq;
    sq.sphere = !(grow_box > 0.0);
    for (int c = 0; c < n_chains && ok; ++c) {
      Region reg;
      if (grow_box > 0.0) {
        const int cx = c % gx, cy = (c / gx) % gy, cz = c / (gx * gy);
        const double edge = grow_box * grow;
        const double ex = edge / gx, ey = edge / gy, ez = edge / gz;
        reg.sphere = false;
        reg.lo = {cx * ex, cy * ey, cz * ez};
        reg.hi = {(cx + 1) * ex, (cy + 1) * ey, (cz + 1) * ez};
        if (compact) {
          // the chain may use the whole cube; its slot only biases the growth
          reg.has_pull = true;
          reg.pull = 0.5 * (reg.lo + reg.hi);
          reg.pull_scale = 0.5 * std::max(ex, std::max(ey, ez));
          reg.lo = {0.0, 0.0, 0.0};
          reg.hi = {edge, edge, edge};
        }
        if (c == 0) {
          sq.lo0 = {0.0, 0.0, 0.0};
          sq.hi0 = {edge, edge, edge};
          const double h = 0.5 * (edge - box_edge);
          sq.lo1 = {h, h, h};
          sq.hi1 = {h + box_edge, h + box_edge, h + box_edge};
        }
      } else {
        reg.sphere = true;
        const double vol = atoms_per_chain / grow_density;
        reg.radius = grow * det::cbrt(3.0 * vol / (4.0 * det::kPi));
        // chains of a multi-chain sphere system are laid side by side along x
        reg.center = {c * (2.0 * reg.radius + 6.0), 0.0, 0.0};
        sq.centre.push_back(reg.center);
        sq.r_start = reg.radius;
        sq.r_target = det::cbrt(3.0 * (atoms_per_chain / density) / (4.0 * det::kPi));
      }
      ok = grow_chain(B, c, n_res, c * n_res, reg, rng);
    }
    if (!ok) continue;
    assemble(B, n_chains, n_res, T);
    if (compact) {
      SqueezeReport rep;
      squeeze(T, B.type, atoms_per_chain, sq, &rep);
      if (squeeze_stats) {
        squeeze_stats[0] = rep.iterations;
        squeeze_stats[1] = rep.max_overlap;
        squeeze_stats[2] = rep.max_outside;
        squeeze_stats[3] = rep.min_nonbonded;
      }
    }
    return true;
  }
  *err = "polyala_build: could not grow the chain(s) without clashes";
  return false;
}

}  // namespace pq
