// C ABI of the GB300 MD step: topology lowering, the batched device arena,
// the per-step launch sequence and its CUDA graph.
//
// Host-side lowering restates the reference engine's constructor
// (NhsAmberFusedEngine::new_on_stream_with_nonbonded_policy,
// crates/prism-nhs/src/fused_engine.rs:10870):
//   exception CSR, both directions, ascending partner       :11625-11680
//   exclusion set = topology exclusions minus exception pairs :11680-11700
//   incidence lists sorted by (term, position)              :11704-11745, :16034-16063
//   H-cluster validation (cardinality, inverse masses, overlap) :11827-11938
//   fixed reference grid from the initial bounding box       :12285-12330
//   Maxwell–Boltzmann start velocities with COM removed      :16065-16100
//
// One step on the device, captured once per batch shape in a CUDA graph:
// the schedule decision (per system) → [control+cells of the rebuilding
// systems → the OU normals → their neighbour rows → their forces] beside
// [the forces of the other systems on a second stream] → integrate
// (post-phases of this step fused with pre-phases of the next).  Systems of
// 16k+ atoms add four grid-wide cell-sort launches after the control kernel.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "pq_common.cuh"
#include "pq_device.cuh"
#include "pq_host.h"

using namespace pq;

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

static prismq_status fail(prismq_status st, const std::string& msg) {
  g_err = msg;
  return st;
}

namespace pq {
// Lets entry points in other translation units report through prismq_last_error().
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace pq

#define PQ_CK(x)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess)                                                                   \
      return fail(PRISMQ_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));           \
  } while (0)

namespace {

// ---------------------------------------------------------------------------
// first-fit range allocator over one arena segment
// ---------------------------------------------------------------------------
struct RangeAlloc {
  int64_t cap = 0;
  std::map<int64_t, int64_t> free_;  // begin -> size
  void init(int64_t c) {
    cap = c;
    free_.clear();
    if (c > 0) free_[0] = c;
  }
  int64_t alloc(int64_t n, int64_t align = 1) {
    if (n == 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      const int64_t b = it->first, sz = it->second;
      const int64_t ab = (b + align - 1) / align * align;
      if (ab + n > b + sz) continue;
      free_.erase(it);
      if (ab > b) free_[b] = ab - b;
      if (b + sz > ab + n) free_[ab + n] = b + sz - (ab + n);
      return ab;
    }
    return -1;
  }
  void release(int64_t b, int64_t n) {
    if (n == 0) return;
    auto it = free_.emplace(b, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  // one past the highest allocated element
  int64_t high() const {
    if (free_.empty()) return cap;
    auto last = std::prev(free_.end());
    return last->first + last->second == cap ? last->first : cap;
  }
};

// ---------------------------------------------------------------------------
// lowered (host, system-local indices) form of one topology
// ---------------------------------------------------------------------------
struct Lowered {
  int n = 0;
  std::vector<float4> pos, vel;
  std::vector<float2> lj;
  std::vector<double2> lj64;  // the same in double (FP64 batches)
  std::vector<unsigned long long> mask_all, mask_ref;
  std::vector<int2> far;
  std::vector<int> far_list;
  std::vector<Incidence> inc;
  std::vector<int> inc_list;  // local term index * 4 + position
  std::vector<int2> ex_idx;
  std::vector<int> ex_partner;
  std::vector<float4> ex_par;
  std::vector<BondT> bonds;
  std::vector<AngleT> angles;
  std::vector<DihT> dihs;
  std::vector<Unit> units;
  std::vector<ExcT> excs;       // exception pairs, each once
  std::vector<int2> grp;        // per 32-atom group: {begin, count} into grp_refs (local)
  std::vector<int> grp_refs;    // kind << 29 | local term index
  int max_group_slots = 0;      // bonded + exception incidences of the fullest group
  std::vector<float> charges, masses;
  float ref_origin[3] = {0, 0, 0};
  int ref_dims[3] = {1, 1, 1};
  bool ref_ok = false;
  int cell_cap = 64;
  uint64_t topo_hash = 0;  // fingerprint of everything but positions and velocities
};

bool finite_pos(float x) { return std::isfinite(x); }

// 64-bit FNV-1a over 8-byte words (then the tail bytes): a fingerprint that
// tells a checkpoint which topology it belongs to.
uint64_t fnv_words(uint64_t h, const void* data, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(data);
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, b + i, 8);
    h = (h ^ w) * 1099511628211ull;
  }
  for (; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  return h;
}
template <class T>
uint64_t fnv_vec(uint64_t h, const std::vector<T>& v) {
  const uint64_t n = v.size();
  h = fnv_words(h, &n, sizeof(n));
  return v.empty() ? h : fnv_words(h, v.data(), sizeof(T) * v.size());
}

uint64_t topology_fingerprint(const Lowered& L) {
  uint64_t h = 14695981039346656037ull;
  h = fnv_words(h, &L.n, sizeof(L.n));
  h = fnv_vec(h, L.charges);
  h = fnv_vec(h, L.masses);
  h = fnv_vec(h, L.lj);
  h = fnv_vec(h, L.mask_all);
  h = fnv_vec(h, L.mask_ref);
  h = fnv_vec(h, L.far);
  h = fnv_vec(h, L.far_list);
  h = fnv_vec(h, L.bonds);
  h = fnv_vec(h, L.angles);
  h = fnv_vec(h, L.dihs);
  h = fnv_vec(h, L.excs);
  h = fnv_vec(h, L.units);
  return h;
}

prismq_status lower_topology(const prismq_topology* T, Lowered* L) {
  if (!T) return fail(PRISMQ_E_INVALID, "topology is NULL");
  const int n = T->n_atoms;
  if (n <= 0) return fail(PRISMQ_E_INVALID, "topology has no atoms");
  if (n > (1 << 29)) return fail(PRISMQ_E_INVALID, "topology exceeds 2^29 atoms");
  if (!T->positions || !T->masses || !T->charges || !T->lj_sigma || !T->lj_epsilon)
    return fail(PRISMQ_E_INVALID, "topology per-atom arrays must be non-NULL");
  L->n = n;
  L->pos.resize(n);
  L->vel.resize(n);
  L->lj.resize(n);
  L->lj64.resize(n);
  L->charges.assign(T->charges, T->charges + n);
  L->masses.assign(T->masses, T->masses + n);
  for (int a = 0; a < n; ++a) {
    const float x = T->positions[3 * a], y = T->positions[3 * a + 1], z = T->positions[3 * a + 2];
    if (!finite_pos(x) || !finite_pos(y) || !finite_pos(z))
      return fail(PRISMQ_E_INVALID, "non-finite position at atom " + std::to_string(a));
    const float m = T->masses[a];
    if (!(m > 0.0f) || !std::isfinite(m))
      return fail(PRISMQ_E_INVALID, "mass must be positive and finite at atom " + std::to_string(a));
    const float sg = T->lj_sigma[a], ep = T->lj_epsilon[a];
    if (!(sg >= 0.0f) || !(ep >= 0.0f) || !std::isfinite(sg) || !std::isfinite(ep) ||
        !std::isfinite(T->charges[a]))
      return fail(PRISMQ_E_INVALID, "invalid charge/LJ parameter at atom " + std::to_string(a));
    L->pos[a] = make_float4(x, y, z, T->charges[a]);
    L->vel[a] = make_float4(0.f, 0.f, 0.f, m);
    L->lj[a] = make_float2(0.5f * sg, sqrtf(ep));
    L->lj64[a] = make_double2(0.5 * (double)sg, std::sqrt((double)ep));
  }
  auto in_range = [n](int i) { return i >= 0 && i < n; };
  // ---- bonded terms + incidence ----
  std::vector<std::vector<int>> ib(n), ia(n), id(n);
  for (int t = 0; t < T->n_bonds; ++t) {
    const prismq_bond& b = T->bonds[t];
    if (!in_range(b.i) || !in_range(b.j) || b.i == b.j)
      return fail(PRISMQ_E_INVALID, "bond " + std::to_string(t) + " has invalid atoms");
    L->bonds.push_back({b.i, b.j, b.r0, b.k, (int)ib[b.i].size() | ((int)ib[b.j].size() << 16)});
    ib[b.i].push_back(t * 4 + 0);
    ib[b.j].push_back(t * 4 + 1);
  }
  for (int t = 0; t < T->n_angles; ++t) {
    const prismq_angle& g = T->angles[t];
    if (!in_range(g.i) || !in_range(g.j) || !in_range(g.k) || g.i == g.j || g.j == g.k || g.i == g.k)
      return fail(PRISMQ_E_INVALID, "angle " + std::to_string(t) + " has invalid atoms");
    // positions past 1023 overflow the packing; such atoms are rejected below (> 255)
    L->angles.push_back({g.i, g.j, g.k, g.theta0, g.force_k,
                         ((int)ia[g.i].size() & 1023) | (((int)ia[g.j].size() & 1023) << 10) |
                             (((int)ia[g.k].size() & 1023) << 20)});
    ia[g.i].push_back(t * 4 + 0);
    ia[g.j].push_back(t * 4 + 1);
    ia[g.k].push_back(t * 4 + 2);
  }
  for (int t = 0; t < T->n_dihedrals; ++t) {
    const prismq_dihedral& d = T->dihedrals[t];
    if (!in_range(d.i) || !in_range(d.j) || !in_range(d.k) || !in_range(d.l))
      return fail(PRISMQ_E_INVALID, "dihedral " + std::to_string(t) + " has invalid atoms");
    // the reference's validate rejects periodicity <= 0 (input.rs:2101); the
    // torsion kernel forms cos and sin of n phi by n steps of a recurrence,
    // so n is also bounded above
    if (d.periodicity < 1 || d.periodicity > kMaxPeriodicity)
      return fail(PRISMQ_E_INVALID, "dihedral " + std::to_string(t) + " has periodicity outside [1, " +
                                        std::to_string(kMaxPeriodicity) + "]");
    L->dihs.push_back({d.i, d.j, d.k, d.l, d.periodicity, d.phase, d.force_k,
                       (float)std::cos((double)d.phase), (float)std::sin((double)d.phase),
                       ((int)id[d.i].size() & 255) | (((int)id[d.j].size() & 255) << 8) |
                           (((int)id[d.k].size() & 255) << 16) | (((int)id[d.l].size() & 255) << 24)});
    id[d.i].push_back(t * 4 + 0);
    id[d.j].push_back(t * 4 + 1);
    id[d.k].push_back(t * 4 + 2);
    id[d.l].push_back(t * 4 + 3);
  }
  if ((int64_t)L->bonds.size() >= (1 << 29) || (int64_t)L->angles.size() >= (1 << 29) ||
      (int64_t)L->dihs.size() >= (1 << 29))
    return fail(PRISMQ_E_INVALID, "too many bonded terms");
  L->inc.resize(n);
  for (int a = 0; a < n; ++a) {
    if (ib[a].size() > 255 || ia[a].size() > 255 || id[a].size() > 255)
      return fail(PRISMQ_E_INVALID, "more than 255 terms of one kind on atom " + std::to_string(a));
    Incidence I;
    I.b_beg = (int)L->inc_list.size();
    L->inc_list.insert(L->inc_list.end(), ib[a].begin(), ib[a].end());
    I.a_beg = (int)L->inc_list.size();
    L->inc_list.insert(L->inc_list.end(), ia[a].begin(), ia[a].end());
    I.d_beg = (int)L->inc_list.size();
    L->inc_list.insert(L->inc_list.end(), id[a].begin(), id[a].end());
    I.counts = (int)ib[a].size() | ((int)ia[a].size() << 8) | ((int)id[a].size() << 16);
    L->inc[a] = I;
  }
  // ---- exceptions (both directions, ascending partner, last definition wins) ----
  std::vector<std::map<int, float4>> exc(n);
  for (int t = 0; t < T->n_exceptions; ++t) {
    const prismq_exception& e = T->exceptions[t];
    if (!in_range(e.i) || !in_range(e.j) || e.i == e.j)
      return fail(PRISMQ_E_INVALID, "exception " + std::to_string(t) + " has invalid atoms");
    if (!std::isfinite(e.charge_product) || !std::isfinite(e.sigma) || !std::isfinite(e.epsilon))
      return fail(PRISMQ_E_INVALID, "exception " + std::to_string(t) + " has non-finite parameters");
    const float4 p = make_float4(e.charge_product, e.sigma, e.epsilon, 0.f);
    exc[e.i][e.j] = p;
    exc[e.j][e.i] = p;
  }
  L->ex_idx.resize(n);
  for (int a = 0; a < n; ++a) {
    if (exc[a].size() > 65535) return fail(PRISMQ_E_INVALID, "too many exceptions on atom " + std::to_string(a));
    L->ex_idx[a] = make_int2((int)L->ex_partner.size(), (int)exc[a].size());
    for (auto& kv : exc[a]) {
      L->ex_partner.push_back(kv.first);
      L->ex_par.push_back(kv.second);
    }
  }
  // each exception pair once, with its rank in both members' ascending lists
  for (int a = 0; a < n; ++a) {
    int ra = 0;
    for (auto& kv : exc[a]) {
      const int j = kv.first;
      if (j > a) {
        const int rj = (int)std::distance(exc[j].begin(), exc[j].find(a));
        L->excs.push_back({a, j, kv.second.x, kv.second.y, kv.second.z, ra | (rj << 16)});
      }
      ++ra;
    }
  }
  // ---- force groups: the terms with a member in each 32-atom group ----
  {
    const int ng = (n + kForceGroup - 1) / kForceGroup;
    std::vector<std::vector<int>> refs(ng);
    auto add = [&](int kind, int t, const int* members, int nm) {
      int last = -1;
      for (int m = 0; m < nm; ++m) {
        const int g = members[m] / kForceGroup;
        bool seen = false;
        for (int q = 0; q < m; ++q) seen = seen || members[q] / kForceGroup == g;
        if (!seen) refs[g].push_back((kind << 29) | t);
        last = g;
      }
      (void)last;
    };
    for (int t = 0; t < (int)L->bonds.size(); ++t) {
      const int mm[2] = {L->bonds[t].i, L->bonds[t].j};
      add(kRefBond, t, mm, 2);
    }
    for (int t = 0; t < (int)L->angles.size(); ++t) {
      const int mm[3] = {L->angles[t].i, L->angles[t].j, L->angles[t].k};
      add(kRefAngle, t, mm, 3);
    }
    for (int t = 0; t < (int)L->dihs.size(); ++t) {
      const int mm[4] = {L->dihs[t].i, L->dihs[t].j, L->dihs[t].k, L->dihs[t].l};
      add(kRefDih, t, mm, 4);
    }
    if ((int64_t)L->excs.size() >= (1 << 29)) return fail(PRISMQ_E_INVALID, "too many exceptions");
    for (int t = 0; t < (int)L->excs.size(); ++t) {
      const int mm[2] = {L->excs[t].i, L->excs[t].j};
      add(kRefExc, t, mm, 2);
    }
    L->grp.resize(ng);
    for (int g = 0; g < ng; ++g) {
      L->grp[g] = make_int2((int)L->grp_refs.size(), (int)refs[g].size());
      L->grp_refs.insert(L->grp_refs.end(), refs[g].begin(), refs[g].end());
      int slots = 0;
      for (int a = g * kForceGroup; a < std::min(n, (g + 1) * kForceGroup); ++a)
        slots += (int)(ib[a].size() + ia[a].size() + id[a].size() + exc[a].size());
      L->max_group_slots = std::max(L->max_group_slots, slots);
    }
    if (L->max_group_slots > kMaxGroupSlots)
      return fail(PRISMQ_E_INVALID, "more than " + std::to_string(kMaxGroupSlots) +
                                        " bonded and exception incidences in one 32-atom group");
  }
  // ---- exclusion window masks ----
  L->mask_all.assign(n, 0ull);
  L->mask_ref.assign(n, 0ull);
  L->far.assign(n, make_int2(0, 0));
  if (T->exclusion_offsets) {
    if (T->exclusion_offsets[0] != 0) return fail(PRISMQ_E_INVALID, "exclusion_offsets[0] must be 0");
    for (int a = 0; a < n; ++a)
      if (T->exclusion_offsets[a + 1] < T->exclusion_offsets[a])
        return fail(PRISMQ_E_INVALID, "exclusion_offsets must be non-decreasing");
    if (T->exclusion_offsets[n] > 0 && !T->exclusions)
      return fail(PRISMQ_E_INVALID, "exclusions array is NULL");
  }
  for (int a = 0; a < n; ++a) {
    std::map<int, int> part;  // partner -> is_exception
    if (T->exclusion_offsets) {
      for (int q = T->exclusion_offsets[a]; q < T->exclusion_offsets[a + 1]; ++q) {
        const int j = T->exclusions[q];
        if (!in_range(j) || j == a)
          return fail(PRISMQ_E_INVALID, "exclusion partner out of range at atom " + std::to_string(a));
        part[j] = exc[a].count(j) ? 1 : 0;
      }
    }
    for (auto& kv : exc[a]) part[kv.first] = 1;  // exception pairs never enter ordinary rows
    const int fb = (int)L->far_list.size();
    for (auto& kv : part) {
      const int d = kv.first - a;
      if (d >= -32 && d < 32) {
        L->mask_all[a] |= 1ull << (d + 32);
        if (!kv.second) L->mask_ref[a] |= 1ull << (d + 32);
      } else {
        L->far_list.push_back(kv.first | (kv.second ? 0x40000000 : 0));
      }
    }
    // an atom excludes itself: the group row builder then needs no separate
    // self test (offset 0 is bit 32 of the window)
    L->mask_all[a] |= 1ull << 32;
    L->mask_ref[a] |= 1ull << 32;
    L->far[a] = make_int2(fb, (int)L->far_list.size() - fb);
  }
  // ---- constraint units (fused_engine.rs:11827-11938) ----
  std::vector<int> owner(n, -1);
  for (int c = 0; c < T->n_clusters; ++c) {
    const prismq_hcluster& h = T->clusters[c];
    const std::string tag = "SHAKE/RATTLE cluster " + std::to_string(c) + ": ";
    if (!in_range(h.central_atom)) return fail(PRISMQ_E_INVALID, tag + "central atom out of range");
    if (h.n_hydrogens < 1 || h.n_hydrogens > 3) return fail(PRISMQ_E_INVALID, tag + "n_hydrogens must be 1..3");
    if (!(h.inv_mass_central > 0.f) || !std::isfinite(h.inv_mass_central) || !(h.inv_mass_h > 0.f) ||
        !std::isfinite(h.inv_mass_h))
      return fail(PRISMQ_E_INVALID, tag + "invalid inverse masses");
    const double live_c = 1.0 / (double)T->masses[h.central_atom];
    if (std::fabs((double)h.inv_mass_central - live_c) / std::max(live_c, 2.2e-16) > 1.0e-6)
      return fail(PRISMQ_E_INVALID, tag + "central inverse mass disagrees with the atom mass");
    if (owner[h.central_atom] >= 0) return fail(PRISMQ_E_INVALID, tag + "clusters overlap");
    owner[h.central_atom] = c;
    Unit U;
    std::memset(&U, 0, sizeof(U));
    U.a[0] = h.central_atom;
    U.a[1] = U.a[2] = U.a[3] = -1;
    U.nh = h.n_hydrogens;
    U.inv_mc = h.inv_mass_central;
    U.inv_mh = h.inv_mass_h;
    for (int q = 0; q < h.n_hydrogens; ++q) {
      const int hq = h.hydrogen_atoms[q];
      if (!in_range(hq) || hq == h.central_atom) return fail(PRISMQ_E_INVALID, tag + "invalid hydrogen atom");
      const float L0 = h.bond_lengths[q];
      if (!(L0 > 0.f) || !std::isfinite(L0)) return fail(PRISMQ_E_INVALID, tag + "invalid bond length");
      const double live_h = 1.0 / (double)T->masses[hq];
      if (std::fabs((double)h.inv_mass_h - live_h) / std::max(live_h, 2.2e-16) > 1.0e-6)
        return fail(PRISMQ_E_INVALID, tag + "hydrogen inverse mass disagrees with the atom mass");
      if (owner[hq] >= 0) return fail(PRISMQ_E_INVALID, tag + "clusters overlap");
      owner[hq] = c;
      U.a[1 + q] = hq;
      U.r0[q] = L0;
    }
    L->units.push_back(U);
  }
  for (int a = 0; a < n; ++a)
    if (owner[a] < 0) {
      Unit U;
      std::memset(&U, 0, sizeof(U));
      U.a[0] = a;
      U.a[1] = U.a[2] = U.a[3] = -1;
      U.nh = 0;
      L->units.push_back(U);
    }
  // Units with the same hydrogen count sit together, so a warp of the
  // integrator runs one control path (no per-atom or constraint divergence).
  std::stable_sort(L->units.begin(), L->units.end(), [](const Unit& x, const Unit& y) {
    return x.nh != y.nh ? x.nh > y.nh : x.a[0] < y.a[0];
  });
  // ---- reference grid (CELL_SIZE 10 Å, one cell of padding, ≤ 32 per axis) ----
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      mn[d] = std::min(mn[d], T->positions[3 * a + d]);
      mx[d] = std::max(mx[d], T->positions[3 * a + d]);
    }
  L->ref_ok = true;
  long long ref_cells = 1;
  for (int d = 0; d < 3; ++d) {
    L->ref_origin[d] = mn[d] - 10.0f;
    const float extent = (mx[d] - mn[d]) + 2.0f * 10.0f;
    long long v = (long long)std::ceil(extent / 10.0f);
    if (v < 1) v = 1;
    if (v > kRefMaxDim) L->ref_ok = false;
    L->ref_dims[d] = (int)std::min<long long>(v, kRefMaxDim);
    ref_cells *= L->ref_dims[d];
  }
  L->cell_cap = (int)std::max<long long>({1024LL, (long long)n / 2, L->ref_ok ? ref_cells : 0LL});
  L->topo_hash = topology_fingerprint(*L);
  return PRISMQ_OK;
}

// Maxwell–Boltzmann velocities: σ_v = sqrt(418.4·k_B·T/m), COM removed.
void init_velocities(Lowered* L, const prismq_params& p) {
  const int n = L->n;
  std::vector<double> vx(n), vy(n), vz(n);
  double px = 0, py = 0, pz = 0, M = 0;
  for (int a = 0; a < n; ++a) {
    const float m = L->vel[a].w;
    float z0 = 0.f, z1 = 0.f, z2 = 0.f;
    if (p.temperature > 0.f) normal3(p.seed, p.stream, (uint32_t)a, 0xffffffffffffull, 3u, &z0, &z1, &z2);
    const float sg = sqrtf(kKcalToAmuA2Ps2 * kBoltzmann * p.temperature / m);
    vx[a] = sg * z0;
    vy[a] = sg * z1;
    vz[a] = sg * z2;
    px += m * vx[a];
    py += m * vy[a];
    pz += m * vz[a];
    M += m;
  }
  for (int a = 0; a < n; ++a) {
    L->vel[a].x = (float)(vx[a] - px / M);
    L->vel[a].y = (float)(vy[a] - py / M);
    L->vel[a].z = (float)(vz[a] - pz / M);
  }
}

prismq_status check_params(const prismq_params* p) {
  if (!p) return fail(PRISMQ_E_INVALID, "params is NULL");
  if (!(p->dt > 0.f) || !std::isfinite(p->dt)) return fail(PRISMQ_E_INVALID, "dt must be positive");
  if (!(p->temperature >= 0.f) || !std::isfinite(p->temperature))
    return fail(PRISMQ_E_INVALID, "temperature must be >= 0");
  if (!(p->gamma >= 0.f) || !std::isfinite(p->gamma)) return fail(PRISMQ_E_INVALID, "gamma must be >= 0");
  if (!(p->cutoff > 0.f) || !(p->skin >= 0.f)) return fail(PRISMQ_E_INVALID, "cutoff/skin invalid");
  if (p->rebuild_interval < 1) return fail(PRISMQ_E_INVALID, "rebuild_interval must be >= 1");
  if (p->max_constraint_iter < 1) return fail(PRISMQ_E_INVALID, "max_constraint_iter must be >= 1");
  if (p->com_interval < 0) return fail(PRISMQ_E_INVALID, "com_interval must be >= 0");
  if (!std::isfinite(p->shake_tol) || !std::isfinite(p->rattle_tol))
    return fail(PRISMQ_E_INVALID, "constraint tolerances must be finite");
  if (p->constraint_check_fp64 != 0 && p->constraint_check_fp64 != 1)
    return fail(PRISMQ_E_INVALID, "constraint_check_fp64 must be 0 or 1");
  if (p->precision != PRISMQ_PRECISION_FP32 && p->precision != PRISMQ_PRECISION_FP64)
    return fail(PRISMQ_E_INVALID, "unknown precision");
  return PRISMQ_OK;
}

// Host-side changes take effect from the next step as a whole: the
// post-force phases still to run belong to that step too.
void carry_post(SysDev* S) {
  S->post_dt = S->dt;
  S->post_temperature = S->temperature;
  S->post_gamma = S->gamma;
  S->post_c1 = S->c1;
  S->post_c1d = S->c1d;
}

// With a protocol installed, the parameters of the next step (S->step) come
// from the director, exactly as the control kernel evaluates them.
void protocol_now(SysDev* S) {
  if (!S->proto.on) return;
  StepParams P;
  protocol_eval(S->proto, S->step - S->proto.origin, &P);
  S->dt = P.dt;
  S->temperature = P.temperature;
  S->gamma = P.gamma;
  S->c1 = P.c1;
  S->c1d = P.c1d;
  carry_post(S);
}

prismq_status check_protocol(const prismq_protocol* p) {
  if (!p) return fail(PRISMQ_E_INVALID, "protocol is NULL");
  auto fin = [](float v) { return std::isfinite(v) && v >= 0.0f; };
  if (!fin(p->start_temp) || !fin(p->end_temp)) return fail(PRISMQ_E_INVALID, "protocol temperatures must be >= 0");
  if (!fin(p->gamma_base) || !fin(p->equilibration_gamma)) return fail(PRISMQ_E_INVALID, "protocol frictions must be >= 0");
  if (!(p->base_dt > 0.0f) || !std::isfinite(p->base_dt)) return fail(PRISMQ_E_INVALID, "protocol base_dt must be positive");
  const int64_t phases[5] = {p->cold_hold_steps, p->ramp_steps, p->warm_hold_steps, p->ramp_down_steps,
                             p->cold_return_steps};
  int64_t total = 0;
  for (int64_t v : phases) {
    if (v < 0) return fail(PRISMQ_E_INVALID, "protocol phase lengths must be >= 0");
    total += v;
  }
  if (total > INT32_MAX) return fail(PRISMQ_E_INVALID, "protocol longer than 2^31-1 steps");
  if (p->equilibration_steps < 0 || p->current_step < 0)
    return fail(PRISMQ_E_INVALID, "protocol equilibration_steps and current_step must be >= 0");
  if (p->adaptive_dt < 0 || p->adaptive_dt > 2) return fail(PRISMQ_E_INVALID, "protocol adaptive_dt must be 0, 1 or 2");
  if (p->cryo_enabled != 0 && p->cryo_enabled != 1) return fail(PRISMQ_E_INVALID, "protocol cryo_enabled must be 0 or 1");
  return PRISMQ_OK;
}

// ProtocolState::from_cryo_uv (protocol_state.rs:602-700): phase ends are
// cumulative; the warm temperature persists when there is no cooling.
ProtocolDev protocol_dev(const prismq_protocol& p, long long origin) {
  ProtocolDev d;
  std::memset(&d, 0, sizeof(d));
  d.on = 1;
  d.adaptive = p.adaptive_dt;
  d.cryo = p.cryo_enabled;
  d.warm_tail = (p.ramp_down_steps == 0 && p.cold_return_steps == 0) ? 1 : 0;
  d.cold_hold_end = p.cold_hold_steps;
  d.ramp_end = d.cold_hold_end + p.ramp_steps;
  d.warm_hold_end = d.ramp_end + p.warm_hold_steps;
  d.ramp_down_end = d.warm_hold_end + p.ramp_down_steps;
  d.equil_steps = p.equilibration_steps;
  d.start_temp = p.start_temp;
  d.end_temp = p.end_temp;
  d.gamma_base = p.gamma_base;
  d.equil_gamma = p.equilibration_gamma;
  d.base_dt = p.base_dt;
  d.origin = origin;
  return d;
}

void fill_params(SysDev* S, const prismq_params& p) {
  S->dt = p.dt;
  S->temperature = p.temperature;
  S->gamma = p.gamma;
  const float hd = 0.5f * p.dt;
  const float arg = -p.gamma * hd;
  S->c1 = (float)std::exp((double)arg);  // exp(-γ·dt/2), rounded once to float
  const float rl = p.cutoff + p.skin;
  S->rlist2 = rl * rl;
  S->half_skin2 = (0.5f * p.skin) * (0.5f * p.skin);
  S->ref_r2 = (p.cutoff * p.cutoff) * 1.44f;
  S->cut2 = p.cutoff * p.cutoff;
  S->rebuild_interval = p.rebuild_interval;
  S->com_interval = p.com_interval;
  S->max_iter = p.max_constraint_iter;
  S->seed = p.seed;
  S->stream = p.stream;
  S->shake_tol = p.shake_tol > 0.f ? p.shake_tol : 1.0e-4f;
  S->rattle_tol = p.rattle_tol > 0.f ? p.rattle_tol : 1.0e-5f;
  S->check64 = p.constraint_check_fp64;
  S->c1d = std::exp(-(double)p.gamma * 0.5 * (double)p.dt);
  carry_post(S);
}

// ---------------------------------------------------------------------------
// small transfer kernels (AoS float[3N] <-> SoA float4 streams)
// ---------------------------------------------------------------------------
__global__ void k_aos_to_xyz(float4* dst, const float* src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 o = dst[i];
  dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], o.w);
}
__global__ void k_xyz_to_aos(float* dst, const float4* src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = src[i];
  dst[3 * i] = v.x;
  dst[3 * i + 1] = v.y;
  dst[3 * i + 2] = v.z;
}
__global__ void k_aos_to_xyz64(double4_32a* dst, const float* src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a o = dst[i];
  dst[i] = make_double4_32a(src[3 * i], src[3 * i + 1], src[3 * i + 2], o.w);
}
__global__ void k_xyz64_to_aos(double* dst, const double4_32a* src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a v = src[i];
  dst[3 * i] = v.x;
  dst[3 * i + 1] = v.y;
  dst[3 * i + 2] = v.z;
}
__global__ void k_xyz_to_aos64(double* dst, const float4* src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = src[i];
  dst[3 * i] = v.x;
  dst[3 * i + 1] = v.y;
  dst[3 * i + 2] = v.z;
}
// Whole-arena state transfer, 256 atoms per block.  The block's AoS segment
// (3072 bytes per array) moves through shared memory as 16-byte vectors when
// the segment is whole and the host-side arrays are 16-byte aligned, so the
// accesses stay contiguous whether the arrays are device staging buffers or
// pinned host memory read and written directly over the host link.
constexpr int kStateBlock = 256;
__device__ __forceinline__ void aos_in(float* dst, const float* src, int64_t a0, int na, bool vec) {
  const int tid = threadIdx.x;
  if (vec && na == kStateBlock) {
    if (tid < 3 * kStateBlock / 4)
      reinterpret_cast<float4*>(dst)[tid] = reinterpret_cast<const float4*>(src + 3 * a0)[tid];
  } else {
    for (int i = tid; i < 3 * na; i += kStateBlock) dst[i] = src[3 * a0 + i];
  }
}
__device__ __forceinline__ void aos_out(float* dst, const float* src, int64_t a0, int na, bool vec) {
  const int tid = threadIdx.x;
  if (vec && na == kStateBlock) {
    if (tid < 3 * kStateBlock / 4)
      reinterpret_cast<float4*>(dst + 3 * a0)[tid] = reinterpret_cast<const float4*>(src)[tid];
  } else {
    for (int i = tid; i < 3 * na; i += kStateBlock) dst[3 * a0 + i] = src[i];
  }
}
// Upload: positions whose bits change mark their system for a force/list
// refresh before the next step.
__global__ void __launch_bounds__(kStateBlock) k_set_state_all(float4* pos, float4* vel, double4_32a* pos64,
                                                               double4_32a* vel64, const float* xs, const float* vs,
                                                               const int* atom_sys, SysDev* sys, int64_t n, int vec) {
  __shared__ __align__(16) float sx[3 * kStateBlock], sv[3 * kStateBlock];
  const int64_t a0 = (int64_t)blockIdx.x * kStateBlock;
  const int na = (int)(n - a0 < kStateBlock ? n - a0 : kStateBlock);
  if (xs) aos_in(sx, xs, a0, na, vec);
  if (vs) aos_in(sv, vs, a0, na, vec);
  __syncthreads();
  const int i = threadIdx.x;
  if (i >= na) return;
  const int64_t a = a0 + i;
  const int s = atom_sys[a];
  if (s < 0) return;
  if (xs) {
    const float4 o = pos[a];
    const float x = sx[3 * i], y = sx[3 * i + 1], z = sx[3 * i + 2];
    if (__float_as_uint(x) != __float_as_uint(o.x) || __float_as_uint(y) != __float_as_uint(o.y) ||
        __float_as_uint(z) != __float_as_uint(o.z)) {
      pos[a] = make_float4(x, y, z, o.w);
      if (pos64) pos64[a] = make_double4_32a(x, y, z, pos64[a].w);
      atomicOr(&sys[s].need_prime, 1);
    }
  }
  if (vs) {
    const float4 o = vel[a];
    const float x = sv[3 * i], y = sv[3 * i + 1], z = sv[3 * i + 2];
    vel[a] = make_float4(x, y, z, o.w);
    if (vel64) vel64[a] = make_double4_32a(x, y, z, vel64[a].w);
  }
}
__global__ void __launch_bounds__(kStateBlock) k_get_state_all(const float4* pos, const float4* vel, float* xs,
                                                               float* vs, int64_t n, int vec) {
  __shared__ __align__(16) float sx[3 * kStateBlock], sv[3 * kStateBlock];
  const int64_t a0 = (int64_t)blockIdx.x * kStateBlock;
  const int na = (int)(n - a0 < kStateBlock ? n - a0 : kStateBlock);
  const int i = threadIdx.x;
  if (i < na) {
    const float4 p = pos[a0 + i], v = vel[a0 + i];
    sx[3 * i] = p.x;
    sx[3 * i + 1] = p.y;
    sx[3 * i + 2] = p.z;
    sv[3 * i] = v.x;
    sv[3 * i + 1] = v.y;
    sv[3 * i + 2] = v.z;
  }
  __syncthreads();
  if (xs) aos_out(xs, sx, a0, na, vec);
  if (vs) aos_out(vs, sv, a0, na, vec);
}
// A host array the kernels may address directly: pinned (page-locked) host
// memory with a device mapping.  Anything else goes through a staging copy.
const float* mapped_host(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // unregistered pageable memory: not an error, just not mapped
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<const float*>(at.devicePointer);
}
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
__global__ void k_fill_int(int* p, int v, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}
__global__ void k_deactivate_units(Unit* u, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) u[i].nh = -1;
}

struct SlotRec {
  bool active = false;
  int64_t atom_b = 0, n_atoms = 0, unit_b = 0, n_units = 0;
  int64_t bond_b = 0, n_bonds = 0, angle_b = 0, n_angles = 0, dih_b = 0, n_dihs = 0;
  int64_t inc_b = 0, n_inc = 0, ex_b = 0, n_ex = 0, far_b = 0, n_far = 0, cell_b = 0, n_cell = 0;
  int64_t exc_b = 0, n_exc = 0, gref_b = 0, n_gref = 0;
  int max_group_slots = 0;
  int32_t units_by_nh[4] = {0, 0, 0, 0};  // the slot's units hold 3, 2, 1, 0 hydrogens in this order
  bool ref_ok = false;
  bool need_prime = true;
  prismq_params params{};
  uint64_t topo_hash = 0;
  // trajectory-frame ring (device memory outside the arena): frame i of the
  // ring holds positions [n_atoms] then, with velocities, [n_atoms] more
  float4* fr_mem = nullptr;
  int fr_interval = 0, fr_cap = 0, fr_vel = 0;
  int64_t fr_written = 0, fr_read = 0;  // frames recorded / handed out so far
  std::vector<int64_t> fr_steps;        // boundary step of each ring entry
};

}  // namespace

struct prismq_batch {
  Arena A;
  RangeAlloc r_atoms, r_units, r_bonds, r_angles, r_dihs, r_inc, r_ex, r_far, r_cells, r_exc, r_gref;
  std::vector<SlotRec> slots;
  cudaStream_t st = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_dirty = true;
  int64_t atom_span = 0, unit_span = 0;
  int sys_span = 0;
  int force_variant = -1;  // autotuned launch shape of the force kernel
  bool force_pinned = false;  // set by prismq_batch_set_force_variant: no re-tuning
  int64_t tuned_span = -1;
  double* d_energy = nullptr;  // kEnergyOut per system
  float* d_stage = nullptr;
  float* d_stage2 = nullptr;
  double* d_stage64 = nullptr;  // allocated on first FP64 read-back
  int precision = PRISMQ_PRECISION_FP32;
  int n_check32 = 0, n_check64 = 0;  // resident FP32 systems by constraint-check precision
  int group_slots = 0;                // the largest force-group slot count among resident systems
  int64_t max_big_atoms = 0;          // the largest resident system of >= kBigSortAtoms atoms (0: none)
  std::vector<SysDev> h_sys;
  // Overlapped step: the branch-B force launch runs on st2 beside the list
  // rebuild on st; st has the higher priority so that the rebuild's few,
  // latency-bound blocks are scheduled ahead of the force launch's many.
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // Host read-back of a step_host call: positions are final once the last
  // step's control kernel has run (a COM step's deferred pre-force phases run
  // there; the post-force phases change velocities only), so the tail graph
  // records ev_xready after it, and st3 (highest priority) packs the
  // positions into the staging buffer and copies them to the host by DMA
  // while the forces and the post-force phases run.
  cudaStream_t st3 = nullptr;
  cudaEvent_t ev_xready = nullptr, ev_xdone = nullptr;

  ~prismq_batch() {
    for (auto& r : slots)
      if (r.fr_mem) cudaFree(r.fr_mem);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (gexec_head) cudaGraphExecDestroy(gexec_head);
    if (gexec_tail) cudaGraphExecDestroy(gexec_tail);
    void* ptrs[] = {A.pos, A.vel, A.lj, A.xref, A.f, A.pe, A.atom_sys, A.mask_all, A.mask_ref, A.far,
                    A.far_list, A.inc, A.inc_list, A.ex_idx, A.ex_partner, A.ex_par, A.exc, A.grp, A.grp_refs, A.bonds, A.angles,
                    A.dihs, A.units, A.order_range, A.order_prefix, A.noise, A.nbr, A.nnbr, A.tiles, A.ntile, A.cell_start, A.cell_atoms, A.atom_cell, A.work, A.work_ctl, A.big_list, A.sys,
                    A.pos64, A.vel64, A.f64, A.lj64, d_energy, d_stage, d_stage2, d_stage64};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_xready) cudaEventDestroy(ev_xready);
    if (ev_xdone) cudaEventDestroy(ev_xdone);
    if (st3) cudaStreamDestroy(st3);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  // The control kernel, followed for large systems by the grid-wide cell sort.
  void control(int mode, int nbr_override, cudaStream_t s) {
    launch_control_cells(A, sys_span, mode, nbr_override, s);
    launch_big_cells(A, max_big_atoms, s);
  }

  // Integrate order: the units of every resident system with three
  // hydrogens, then two, one and none.  The integrate grid walks this list,
  // so the longest constraint chains start in the first wave of blocks and
  // the short ones fill in behind them.  Each unit is still integrated once,
  // by the same code, so the order changes no result.
  // The order is uploaded as 4 ranges per system slot (a few kB), not as one
  // index per unit, so admitting or removing a system costs a small copy.
  std::vector<int2> h_range;
  std::vector<int> h_prefix;
  int64_t n_order = 0;
  prismq_status upload_order() {
    const int nr = 4 * sys_span;
    h_range.assign((size_t)nr, make_int2(0, 0));
    h_prefix.assign((size_t)nr + 1, 0);
    int64_t acc = 0;
    int k = 0;
    for (int nh = 3; nh >= 0; --nh)
      for (int i = 0; i < sys_span; ++i, ++k) {
        const SlotRec& R = slots[i];
        int64_t b = R.unit_b;
        for (int q = 3; q > nh; --q) b += R.units_by_nh[3 - q];
        const int cnt = R.active ? R.units_by_nh[3 - nh] : 0;
        h_range[k] = make_int2((int)b, cnt);
        h_prefix[k] = (int)acc;
        acc += cnt;
      }
    h_prefix[nr] = (int)acc;
    if (acc != n_order || nr != A.n_ranges) graph_dirty = true;
    n_order = acc;
    A.n_ranges = nr;
    if (nr > 0) {
      PQ_CK(cudaMemcpyAsync(A.order_range, h_range.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice, st));
      PQ_CK(cudaMemcpyAsync(A.order_prefix, h_prefix.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice, st));
    }
    return PRISMQ_OK;
  }

  // The step's row builder walks its queue round-robin once more than two
  // systems are resident (it then runs beside the other systems' forces);
  // otherwise its warps take groups from a shared counter.
  bool build_round_robin = false;

  void update_spans() {
    const int64_t na = r_atoms.high(), nu = r_units.high();
    int ns = 0;
    int c32 = 0, c64 = 0;
    int gs = 0;
    int64_t big = 0;
    for (int i = 0; i < (int)slots.size(); ++i)
      if (slots[i].active) {
        if (slots[i].n_atoms >= kBigSortAtoms) big = std::max(big, slots[i].n_atoms);
        ns = i + 1;
        (slots[i].params.constraint_check_fp64 ? c64 : c32) += 1;
        gs = std::max(gs, slots[i].max_group_slots);
      }
    if (gs != group_slots) graph_dirty = true;
    group_slots = gs;
    if (big != max_big_atoms) graph_dirty = true;
    max_big_atoms = big;
    if (na != atom_span || nu != unit_span || ns != sys_span) graph_dirty = true;
    if ((c32 > 0) != (n_check32 > 0) || (c64 > 0) != (n_check64 > 0)) graph_dirty = true;
    int resident = 0;
    for (const SlotRec& R : slots) resident += R.active ? 1 : 0;
    if ((resident > 2) != build_round_robin) graph_dirty = true;
    build_round_robin = resident > 2;
    n_check32 = c32;
    n_check64 = c64;
    atom_span = na;
    unit_span = nu;
    sys_span = ns;
  }

  prismq_status sync_sys_from_device() {
    if (sys_span == 0) return PRISMQ_OK;
    PQ_CK(cudaMemcpyAsync(h_sys.data(), A.sys, sizeof(SysDev) * sys_span, cudaMemcpyDeviceToHost, st));
    PQ_CK(cudaStreamSynchronize(st));
    return PRISMQ_OK;
  }

  // The integrate launch(es) of one step, after the OU normals (drawn here
  // unless the step body already drew them): FP64 batches run one pass; FP32
  // batches run one pass per constraint-check precision present.  Returns the
  // number of kernels launched.
  int integrate(int mode, bool noise = true) {
    if (noise) launch_noise(A, atom_span, mode, st);
    if (A.fp64) {
      launch_integrate(A, n_order, mode, st, 0);
      return noise ? 2 : 1;
    }
    int k = noise ? 1 : 0;
    if (n_check32 > 0 || n_check64 == 0) {
      launch_integrate(A, n_order, mode, st, 0);
      ++k;
    }
    if (n_check64 > 0) {
      launch_integrate(A, n_order, mode, st, 1);
      ++k;
    }
    return k;
  }
  int integrate_passes() const {
    return 1 + (A.fp64 ? 1 : (n_check32 > 0 || n_check64 == 0 ? 1 : 0) + (n_check64 > 0 ? 1 : 0));
  }

  // One step up to its forces.  k_decide chooses the systems that rebuild
  // their lists (or remove their COM velocity) this step; on st their cells
  // are sorted, their rows built and their forces evaluated, while on st2 the
  // forces of every other system, which need none of that, are evaluated at
  // the same time.  (Sorting the cells before the fork, on an empty GPU, was
  // measured slower: 0.93 against 0.84 ms per step on 256 systems.)  Each system's forces come from exactly one of the two
  // force launches, with the same code, so the results do not depend on the
  // split.
  // ev (optional, 4 events, captured as external records): before k_decide,
  // after the control kernel, after the row builder, after the join.
  // evb (optional, 2): around the branch-B force launch on st2.
  // xready (optional, captured as an external record): after the control
  // kernel, when every position of the step is final.
  // The OU normals of the step's integrate launch (mode) are drawn on st
  // right after the control kernel: they need only the step's decisions, so
  // they run beside the forces instead of after the join.
  prismq_status enqueue_step_body(int mode, cudaEvent_t* ev = nullptr, cudaEvent_t* evb = nullptr,
                                  cudaEvent_t xready = nullptr) {
    if (ev) PQ_CK(cudaEventRecordWithFlags(ev[0], st, cudaEventRecordExternal));
    launch_decide(A, sys_span, st);
    PQ_CK(cudaEventRecord(ev_fork, st));
    PQ_CK(cudaStreamWaitEvent(st2, ev_fork, 0));
    if (evb) PQ_CK(cudaEventRecordWithFlags(evb[0], st2, cudaEventRecordExternal));
    launch_force(A, atom_span, false, st2, kSelBranchB, force_variant, group_slots);
    if (evb) PQ_CK(cudaEventRecordWithFlags(evb[1], st2, cudaEventRecordExternal));
    control(kCtlStep, -1, st);
    if (xready) PQ_CK(cudaEventRecordWithFlags(xready, st, cudaEventRecordExternal));
    launch_noise(A, atom_span, mode, st);
    if (ev) PQ_CK(cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal));
    launch_nbr_build(A, atom_span, 1, st, build_round_robin);
    if (ev) PQ_CK(cudaEventRecordWithFlags(ev[2], st, cudaEventRecordExternal));
    launch_force(A, atom_span, false, st, kSelBranchA, force_variant, group_slots);
    PQ_CK(cudaEventRecord(ev_join, st2));
    PQ_CK(cudaStreamWaitEvent(st, ev_join, 0));
    if (ev) PQ_CK(cudaEventRecordWithFlags(ev[3], st, cudaEventRecordExternal));
    return PRISMQ_OK;
  }
  int body_launches() const { return 5 + (max_big_atoms > 0 ? 4 : 0); }

  // Autotuner: time every force-kernel launch shape on the resident batch
  // (three launches each, CUDA events) and keep the fastest.  The shapes give
  // identical forces, so the choice affects speed only.
  prismq_status tune_force() {
    // re-tune only when the resident span has changed by 2x or more since the
    // last tuning, so that admission churn in a server does not re-time shapes
    if (force_pinned) return PRISMQ_OK;
    if (force_variant >= 0 && atom_span <= 2 * tuned_span && 2 * atom_span >= tuned_span) return PRISMQ_OK;
    cudaEvent_t e0, e1;
    PQ_CK(cudaEventCreate(&e0));
    PQ_CK(cudaEventCreate(&e1));
    float best = 3.4e38f;
    int pick = 0;
    for (int v = 0; v < force_variant_count(); ++v) {
      launch_force(A, atom_span, false, st, kSelAll, v, group_slots);
      PQ_CK(cudaEventRecord(e0, st));
      for (int r = 0; r < 3; ++r) launch_force(A, atom_span, false, st, kSelAll, v, group_slots);
      PQ_CK(cudaEventRecord(e1, st));
      PQ_CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      PQ_CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        pick = v;
      }
      g_launches += 4;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    PQ_CK(cudaGetLastError());
    force_variant = pick;
    tuned_span = atom_span;
    return PRISMQ_OK;
  }

  // Three graphs per batch shape: the head of a call (pre-force phases of its
  // first step), the steady step, and the tail (the last step's forces and
  // post-force phases), so that even a one-step call is two graph launches.
  prismq_status capture(int part, cudaGraphExec_t* out) {
    cudaGraph_t g;
    PQ_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    prismq_status brc = PRISMQ_OK;
    if (part == 0) {
      integrate(kIntPre);
    } else {
      const int mode = part == 1 ? kIntBoth : kIntPost;
      brc = enqueue_step_body(mode, nullptr, nullptr, part == 2 ? ev_xready : nullptr);
      integrate(mode, false);
    }
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (brc != PRISMQ_OK) return brc;
    PQ_CK(ce);
    cudaError_t e = cudaGraphInstantiateWithFlags(out, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    PQ_CK(e);
    return PRISMQ_OK;
  }

  prismq_status ensure_graph() {
    prismq_status trc = tune_force();
    if (trc != PRISMQ_OK) return trc;
    if (!graph_dirty && gexec) return PRISMQ_OK;
    for (cudaGraphExec_t* g : {&gexec, &gexec_head, &gexec_tail})
      if (*g) {
        cudaGraphExecDestroy(*g);
        *g = nullptr;
      }
    if ((trc = capture(1, &gexec)) != PRISMQ_OK) return trc;
    if ((trc = capture(0, &gexec_head)) != PRISMQ_OK) return trc;
    if ((trc = capture(2, &gexec_tail)) != PRISMQ_OK) return trc;
    graph_dirty = false;
    return PRISMQ_OK;
  }
  cudaGraphExec_t gexec_head = nullptr, gexec_tail = nullptr;

  prismq_status prime_if_needed() {
    bool any = false;
    for (auto& s : slots)
      if (s.active && s.need_prime) any = true;
    if (!any) return PRISMQ_OK;
    return prime_flagged();
  }

  // Refresh lists and forces of the systems whose device need_prime flag is set.
  prismq_status prime_flagged() {
    control(kCtlPrime, -1, st);
    launch_nbr_build(A, atom_span, 1, st);
    launch_force(A, atom_span, false, st, kSelRebuilding, 0, group_slots);
    g_launches += 3 + (max_big_atoms > 0 ? 4 : 0);
    PQ_CK(cudaGetLastError());
    for (auto& s : slots) s.need_prime = false;
    return PRISMQ_OK;
  }

  prismq_status check_status(int only_slot = -1) {
    prismq_status rc = sync_sys_from_device();
    if (rc != PRISMQ_OK) return rc;
    for (int i = 0; i < sys_span; ++i) {
      if (!slots[i].active) continue;
      if (only_slot >= 0 && i != only_slot) continue;
      const int stt = h_sys[i].status;
      if (stt) return status_error(stt, i);
    }
    return PRISMQ_OK;
  }

  static prismq_status status_error(int stt, int slot) {
    const std::string where = " (system slot " + std::to_string(slot) + ")";
    if (stt & kStShake) return fail(PRISMQ_E_SHAKE, "SHAKE did not converge" + where);
    if (stt & kStRattle) return fail(PRISMQ_E_RATTLE, "RATTLE did not converge" + where);
    if (stt & kStCellOverflow) return fail(PRISMQ_E_CELL_OVERFLOW, "cell occupancy above 512" + where);
    if (stt & kStNbrOverflow)
      return fail(PRISMQ_E_NEIGHBOR_OVERFLOW,
                  "neighbour list above capacity (a row above 1024, or above 768 tiles per 8-atom cluster)" + where);
    return fail(PRISMQ_E_NONFINITE, "non-finite state" + where);
  }

  // n steady steps captured in one graph with events between the launches;
  // head and tail phases run outside the timed graph.
  // phase_ms (optional, 5*n entries): for step i the device time of
  // [decide + control + OU normals, row builder, branch-A forces up to the
  // join, integrate] on the main stream, then the branch-B force launch on
  // the second stream (which overlaps the first three).
  prismq_status run_timed(int64_t n, float* total_ms, float* phase_ms) {
    if (n <= 0 || sys_span == 0) return fail(PRISMQ_E_INVALID, "nothing to time");
    prismq_status rc = prime_if_needed();
    if (rc != PRISMQ_OK) return rc;
    if ((rc = tune_force()) != PRISMQ_OK) return rc;
    std::vector<cudaEvent_t> ev(4 * n + 1), evb(2 * n);
    for (auto& e : ev) PQ_CK(cudaEventCreate(&e));
    for (auto& e : evb) PQ_CK(cudaEventCreate(&e));
    g_launches += integrate(kIntPre);
    cudaGraph_t g;
    cudaGraphExec_t ge = nullptr;
    PQ_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    prismq_status brc = PRISMQ_OK;
    for (int64_t i = 0; i < n && brc == PRISMQ_OK; ++i) {
      brc = enqueue_step_body(kIntBoth, &ev[4 * i], &evb[2 * i]);
      integrate(kIntBoth, false);
    }
    cudaEventRecordWithFlags(ev[4 * n], st, cudaEventRecordExternal);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (brc != PRISMQ_OK) return brc;
    PQ_CK(ce);
    cudaError_t e = cudaGraphInstantiateWithFlags(&ge, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    PQ_CK(e);
    PQ_CK(cudaStreamSynchronize(st));
    nvtxRangePushA("prismq_timed");  // profilers can restrict capture to this range
    cudaError_t le = cudaGraphLaunch(ge, st);
    nvtxRangePop();
    PQ_CK(le);
    g_launches += (body_launches() + integrate_passes()) * n;
    PQ_CK(cudaStreamSynchronize(st));
    PQ_CK(cudaEventElapsedTime(total_ms, ev[0], ev[4 * n]));
    if (phase_ms)
      for (int64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 4; ++k) PQ_CK(cudaEventElapsedTime(&phase_ms[5 * i + k], ev[4 * i + k], ev[4 * i + k + 1]));
        PQ_CK(cudaEventElapsedTime(&phase_ms[5 * i + 4], evb[2 * i], evb[2 * i + 1]));
      }
    cudaGraphExecDestroy(ge);
    for (auto& x : ev) cudaEventDestroy(x);
    for (auto& x : evb) cudaEventDestroy(x);
    if ((rc = enqueue_step_body(kIntPost)) != PRISMQ_OK) return rc;
    g_launches += body_launches() + 1 + integrate(kIntPost, false);
    PQ_CK(cudaGetLastError());
    return check_status();
  }

  // The force kernel over every resident system, timed alone: n launches
  // between two events on the main stream.
  prismq_status time_force(int n, float* ms_per_launch) {
    if (n <= 0 || sys_span == 0) return fail(PRISMQ_E_INVALID, "nothing to time");
    prismq_status rc = prime_if_needed();
    if (rc != PRISMQ_OK) return rc;
    if ((rc = tune_force()) != PRISMQ_OK) return rc;
    cudaEvent_t e0, e1;
    PQ_CK(cudaEventCreate(&e0));
    PQ_CK(cudaEventCreate(&e1));
    launch_force(A, atom_span, false, st, kSelAll, force_variant, group_slots);  // warm
    PQ_CK(cudaEventRecord(e0, st));
    for (int i = 0; i < n; ++i) launch_force(A, atom_span, false, st, kSelAll, force_variant, group_slots);
    PQ_CK(cudaEventRecord(e1, st));
    PQ_CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    PQ_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_launches += n + 1;
    *ms_per_launch = ms / (float)n;
    return PRISMQ_OK;
  }

  // Steps in segments that end on every trajectory-frame boundary of the
  // resident systems; after each segment the systems at a boundary copy their
  // state into their rings.  A segment ends with the post-force phases, which
  // is where any call of step() ends, so results do not depend on the frames.
  prismq_status step_with_frames(int64_t n) {
    prismq_status rc = sync_sys_from_device();
    if (rc != PRISMQ_OK) return rc;
    prismq_status first_failure = PRISMQ_OK;  // a failed system freezes; the others run on
    while (n > 0) {
      int64_t m = n;
      for (int i = 0; i < sys_span; ++i) {
        const SlotRec& R = slots[i];
        if (!R.active || R.fr_interval <= 0 || h_sys[i].status != 0) continue;
        m = std::min<int64_t>(m, R.fr_interval - h_sys[i].step % R.fr_interval);
      }
      rc = step_segment(m);
      if (rc == PRISMQ_E_SHAKE || rc == PRISMQ_E_RATTLE || rc == PRISMQ_E_NONFINITE || rc == PRISMQ_E_CELL_OVERFLOW ||
          rc == PRISMQ_E_NEIGHBOR_OVERFLOW) {
        if (first_failure == PRISMQ_OK) first_failure = rc;
      } else if (rc != PRISMQ_OK) {
        return rc;
      }
      for (int i = 0; i < sys_span; ++i) {  // h_sys was refreshed by the status check
        SlotRec& R = slots[i];
        const SysDev& S = h_sys[i];
        if (!R.active || R.fr_interval <= 0 || S.status != 0 || S.step % R.fr_interval != 0) continue;
        if (R.fr_written > 0 && R.fr_steps[(R.fr_written - 1) % R.fr_cap] == S.step) continue;
        const int64_t slot = R.fr_written % R.fr_cap;
        const size_t plane = sizeof(float4) * (size_t)R.n_atoms;
        float4* dst = R.fr_mem + slot * (R.fr_vel ? 2 : 1) * R.n_atoms;
        PQ_CK(cudaMemcpyAsync(dst, A.pos + R.atom_b, plane, cudaMemcpyDeviceToDevice, st));
        if (R.fr_vel) PQ_CK(cudaMemcpyAsync(dst + R.n_atoms, A.vel + R.atom_b, plane, cudaMemcpyDeviceToDevice, st));
        R.fr_steps[slot] = S.step;
        R.fr_written += 1;
      }
      n -= m;
    }
    return first_failure;
  }

  prismq_status step(int64_t n) {
    if (n <= 0) return PRISMQ_OK;
    if (sys_span == 0) return PRISMQ_OK;
    for (int i = 0; i < sys_span; ++i)
      if (slots[i].active && slots[i].fr_interval > 0) return step_with_frames(n);
    return step_segment(n);
  }

  // `check` false: the launches are enqueued and the status check is left to
  // the caller (prismq_batch_step_host reads the status with the state).
  prismq_status step_segment(int64_t n, bool check = true) {
    prismq_status rc = prime_if_needed();
    if (rc != PRISMQ_OK) return rc;
    rc = ensure_graph();
    if (rc != PRISMQ_OK) return rc;
    const int per_step = body_launches() + integrate_passes();
    PQ_CK(cudaGraphLaunch(gexec_head, st));
    for (int64_t i = 1; i < n; ++i) PQ_CK(cudaGraphLaunch(gexec, st));
    PQ_CK(cudaGraphLaunch(gexec_tail, st));
    g_launches += (int64_t)per_step * n + integrate_passes();  // head: the noise and integrate launches once more
    PQ_CK(cudaGetLastError());
    return check ? check_status() : PRISMQ_OK;
  }

  bool recording_frames() const {
    for (int i = 0; i < sys_span; ++i)
      if (slots[i].active && slots[i].fr_interval > 0) return true;
    return false;
  }
};

struct prismq_system {
  prismq_batch* b = nullptr;
  int slot = 0;
};

namespace {

// Allocate the arena.  With `dry` set nothing touches the device: *bytes_out
// receives the device bytes the same call would allocate.
prismq_status batch_alloc(prismq_batch* B, int64_t atom_cap, int sys_cap, int64_t bond_cap,
                          int64_t angle_cap, int64_t dih_cap, int64_t inc_cap, int64_t ex_cap,
                          int64_t far_cap, int64_t cell_cap, int64_t exc_cap, int64_t gref_cap,
                          int precision = PRISMQ_PRECISION_FP32,
                          bool dry = false, int64_t* bytes_out = nullptr) {
  int ndev = 0;
  if (!dry && (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)) {
    cudaGetLastError();
    return fail(PRISMQ_E_NO_DEVICE, "no CUDA device visible");
  }
  int64_t total = 0;
  atom_cap = (atom_cap + 31) / 32 * 32;
  Arena& A = B->A;
  A.atom_cap = atom_cap;
  A.unit_cap = atom_cap;
  A.bond_cap = std::max<int64_t>(bond_cap, 1);
  A.angle_cap = std::max<int64_t>(angle_cap, 1);
  A.dih_cap = std::max<int64_t>(dih_cap, 1);
  A.inc_cap = std::max<int64_t>(inc_cap, 1);
  A.ex_cap = std::max<int64_t>(ex_cap, 1);
  A.far_cap = std::max<int64_t>(far_cap, 1);
  A.cell_cap = std::max<int64_t>(cell_cap, 1);
  A.exc_cap = std::max<int64_t>(exc_cap, 1);
  A.gref_cap = std::max<int64_t>(gref_cap, 1);
  A.sys_cap = sys_cap;
  if (!dry) {
    int lo = 0, hi = 0;
    PQ_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PQ_CK(cudaStreamCreateWithPriority(&B->st, cudaStreamNonBlocking, hi));
    PQ_CK(cudaStreamCreateWithPriority(&B->st2, cudaStreamNonBlocking, lo));
    PQ_CK(cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming));
    PQ_CK(cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming));
    PQ_CK(cudaStreamCreateWithPriority(&B->st3, cudaStreamNonBlocking, hi));
    PQ_CK(cudaEventCreateWithFlags(&B->ev_xready, cudaEventDisableTiming));
    PQ_CK(cudaEventCreateWithFlags(&B->ev_xdone, cudaEventDisableTiming));
  }
#define PQ_ALLOC(ptr, count)                                  \
  do {                                                        \
    const size_t nb_ = sizeof(*(ptr)) * (size_t)(count);      \
    total += (int64_t)nb_;                                    \
    if (!dry) PQ_CK(cudaMalloc((void**)&(ptr), nb_));         \
  } while (0)
  PQ_ALLOC(A.pos, atom_cap);
  PQ_ALLOC(A.vel, atom_cap);
  PQ_ALLOC(A.lj, atom_cap);
  PQ_ALLOC(A.xref, atom_cap);
  PQ_ALLOC(A.f, 3 * atom_cap);
  PQ_ALLOC(A.pe, 5 * atom_cap);
  PQ_ALLOC(A.atom_sys, atom_cap);
  PQ_ALLOC(A.mask_all, atom_cap);
  PQ_ALLOC(A.mask_ref, atom_cap);
  PQ_ALLOC(A.far, atom_cap);
  PQ_ALLOC(A.far_list, A.far_cap);
  PQ_ALLOC(A.inc, atom_cap);
  PQ_ALLOC(A.inc_list, A.inc_cap);
  PQ_ALLOC(A.ex_idx, atom_cap);
  PQ_ALLOC(A.ex_partner, A.ex_cap);
  PQ_ALLOC(A.ex_par, A.ex_cap);
  PQ_ALLOC(A.exc, A.exc_cap);
  PQ_ALLOC(A.grp, atom_cap / kForceGroup + 1);
  PQ_ALLOC(A.grp_refs, A.gref_cap);
  PQ_ALLOC(A.bonds, A.bond_cap);
  PQ_ALLOC(A.angles, A.angle_cap);
  PQ_ALLOC(A.dihs, A.dih_cap);
  PQ_ALLOC(A.units, A.unit_cap);
  PQ_ALLOC(A.order_range, 4 * (int64_t)sys_cap);
  PQ_ALLOC(A.order_prefix, 4 * (int64_t)sys_cap + 1);
  PQ_ALLOC(A.noise, 2 * atom_cap);
  PQ_ALLOC(A.nbr, (atom_cap / 32) * (int64_t)kNbrCap * 32);
  PQ_ALLOC(A.nnbr, atom_cap);
  PQ_ALLOC(A.tiles, (atom_cap / 8) * (int64_t)kTileCap);
  PQ_ALLOC(A.ntile, atom_cap / 8 + 1);
  PQ_ALLOC(A.cell_start, A.cell_cap);
  PQ_ALLOC(A.cell_atoms, atom_cap);
  PQ_ALLOC(A.atom_cell, atom_cap);
  PQ_ALLOC(A.work, atom_cap / 8 + sys_cap + 1);
  PQ_ALLOC(A.big_list, sys_cap);
  PQ_ALLOC(A.work_ctl, 4);
  PQ_ALLOC(A.sys, sys_cap);
  PQ_ALLOC(B->d_energy, kEnergyOut * (int64_t)sys_cap);
  if (precision == PRISMQ_PRECISION_FP64) {
    PQ_ALLOC(A.pos64, atom_cap);
    PQ_ALLOC(A.vel64, atom_cap);
    PQ_ALLOC(A.f64, 3 * atom_cap);
    PQ_ALLOC(A.lj64, atom_cap);
  }
  PQ_ALLOC(B->d_stage, 3 * atom_cap);
  PQ_ALLOC(B->d_stage2, 3 * atom_cap);
#undef PQ_ALLOC
  if (bytes_out) *bytes_out = total;
  if (dry) return PRISMQ_OK;
  B->precision = precision;
  A.fp64 = precision == PRISMQ_PRECISION_FP64 ? 1 : 0;
  if (A.fp64) PQ_CK(cudaMemsetAsync(A.f64, 0, sizeof(double) * 3 * atom_cap, B->st));
  PQ_CK(cudaMemsetAsync(A.sys, 0, sizeof(SysDev) * sys_cap, B->st));
  PQ_CK(cudaMemsetAsync(A.nnbr, 0, sizeof(int) * atom_cap, B->st));
  PQ_CK(cudaMemsetAsync(A.ntile, 0, sizeof(int) * (atom_cap / 8 + 1), B->st));
  PQ_CK(cudaMemsetAsync(A.grp, 0, sizeof(int2) * (atom_cap / kForceGroup + 1), B->st));
  PQ_CK(cudaMemsetAsync(A.work_ctl, 0, sizeof(int) * 4, B->st));
  PQ_CK(cudaMemsetAsync(A.f, 0, sizeof(long long) * 3 * atom_cap, B->st));
  PQ_CK(cudaMemsetAsync(A.pe, 0, sizeof(double) * 5 * atom_cap, B->st));
  k_fill_int<<<(unsigned)((atom_cap + 255) / 256), 256, 0, B->st>>>(A.atom_sys, -1, atom_cap);
  k_deactivate_units<<<(unsigned)((atom_cap + 255) / 256), 256, 0, B->st>>>(A.units, atom_cap);
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaStreamSynchronize(B->st));
  B->r_atoms.init(atom_cap);
  B->r_units.init(atom_cap);
  B->r_bonds.init(A.bond_cap);
  B->r_angles.init(A.angle_cap);
  B->r_dihs.init(A.dih_cap);
  B->r_inc.init(A.inc_cap);
  B->r_ex.init(A.ex_cap);
  B->r_far.init(A.far_cap);
  B->r_cells.init(A.cell_cap);
  B->r_exc.init(A.exc_cap);
  B->r_gref.init(A.gref_cap);
  B->slots.resize(sys_cap);
  B->h_sys.resize(sys_cap);
  return PRISMQ_OK;
}

// Arena capacities of a batch for max_atoms atoms in max_systems systems:
// per-atom term capacities cover poly-peptide topologies with margin (bonds
// 2/atom, angles 4, torsion terms 8, incidence entries 48, exceptions 8, far
// exclusions 2) and every system may pad its atom range to 32.
prismq_status batch_alloc_sized(prismq_batch* B, int64_t max_atoms, int32_t max_systems, bool dry,
                                int64_t* bytes_out, int precision = PRISMQ_PRECISION_FP32) {
  const int64_t na = (max_atoms + 31) / 32 * 32 + 32 * (int64_t)max_systems;
  return batch_alloc(B, na, max_systems, 2 * na, 4 * na, 8 * na, 48 * na, 8 * na, 2 * na,
                     2 * (na / 2 + 1026 * (int64_t)max_systems), 4 * na, 16 * na, precision, dry, bytes_out);
}

template <class T>
prismq_status upload(T* dst, const std::vector<T>& src, cudaStream_t st) {
  if (src.empty()) return PRISMQ_OK;
  PQ_CK(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, st));
  return PRISMQ_OK;
}

prismq_status batch_admit(prismq_batch* B, const Lowered& L0, const prismq_params& p, int* slot_out) {
  int slot = -1;
  for (int i = 0; i < (int)B->slots.size(); ++i)
    if (!B->slots[i].active) {
      slot = i;
      break;
    }
  if (slot < 0) return fail(PRISMQ_E_CAPACITY, "batch has no free system slot");
  if (p.precision != B->precision)
    return fail(PRISMQ_E_INVALID, "params.precision differs from the batch's precision");
  Lowered L = L0;
  SlotRec R;
  R.n_atoms = L.n;
  R.n_units = (int64_t)L.units.size();
  R.n_bonds = (int64_t)L.bonds.size();
  R.n_angles = (int64_t)L.angles.size();
  R.n_dihs = (int64_t)L.dihs.size();
  R.n_inc = (int64_t)L.inc_list.size();
  R.n_ex = (int64_t)L.ex_partner.size();
  R.n_far = (int64_t)L.far_list.size();
  R.n_cell = 2 * ((int64_t)L.cell_cap + 1);
  R.n_exc = (int64_t)L.excs.size();
  R.n_gref = (int64_t)L.grp_refs.size();
  R.max_group_slots = L.max_group_slots;
  struct Req {
    RangeAlloc* r;
    int64_t n;
    int64_t* b;
    int64_t align;
  } reqs[] = {{&B->r_atoms, R.n_atoms, &R.atom_b, 32}, {&B->r_units, R.n_units, &R.unit_b, 1},
              {&B->r_bonds, R.n_bonds, &R.bond_b, 1},  {&B->r_angles, R.n_angles, &R.angle_b, 1},
              {&B->r_dihs, R.n_dihs, &R.dih_b, 1},     {&B->r_inc, R.n_inc, &R.inc_b, 1},
              {&B->r_ex, R.n_ex, &R.ex_b, 1},          {&B->r_far, R.n_far, &R.far_b, 1},
              {&B->r_cells, R.n_cell, &R.cell_b, 1},   {&B->r_exc, R.n_exc, &R.exc_b, 1},
              {&B->r_gref, R.n_gref, &R.gref_b, 1}};
  int done = 0;
  for (auto& q : reqs) {
    const int64_t b = q.r->alloc(q.n, q.align);
    if (b < 0) {
      for (int k = 0; k < done; ++k) reqs[k].r->release(*reqs[k].b, reqs[k].n);
      return fail(PRISMQ_E_CAPACITY, "batch arena has no room for this system");
    }
    *q.b = b;
    ++done;
  }
  const int ab = (int)R.atom_b;
  // globalise indices
  for (auto& b : L.bonds) {
    b.i += ab;
    b.j += ab;
  }
  for (auto& g : L.angles) {
    g.i += ab;
    g.j += ab;
    g.k += ab;
  }
  for (auto& d : L.dihs) {
    d.i += ab;
    d.j += ab;
    d.k += ab;
    d.l += ab;
  }
  for (int a = 0; a < L.n; ++a) {
    Incidence& I = L.inc[a];
    const int nb = I.counts & 0xff, na = (I.counts >> 8) & 0xff, nd = (I.counts >> 16) & 0xff;
    for (int q = 0; q < nb; ++q) L.inc_list[I.b_beg + q] += (int)R.bond_b * 4;
    for (int q = 0; q < na; ++q) L.inc_list[I.a_beg + q] += (int)R.angle_b * 4;
    for (int q = 0; q < nd; ++q) L.inc_list[I.d_beg + q] += (int)R.dih_b * 4;
    I.b_beg += (int)R.inc_b;
    I.a_beg += (int)R.inc_b;
    I.d_beg += (int)R.inc_b;
    L.ex_idx[a].x += (int)R.ex_b;
    L.far[a].x += (int)R.far_b;
  }
  for (auto& j : L.ex_partner) j += ab;
  for (auto& e : L.excs) {
    e.i += ab;
    e.j += ab;
  }
  for (auto& r : L.grp_refs) {
    const int kind = r >> 29, t = r & ((1 << 29) - 1);
    const int64_t base = kind == kRefBond ? R.bond_b : kind == kRefAngle ? R.angle_b : kind == kRefDih ? R.dih_b : R.exc_b;
    r = (kind << 29) | (int)(t + base);
  }
  for (auto& g : L.grp) g.x += (int)R.gref_b;
  for (auto& e : L.far_list) e = ((e & 0x3fffffff) + ab) | (e & 0x40000000);
  for (auto& U : L.units) {
    for (int k = 0; k < 4; ++k)
      if (U.a[k] >= 0) U.a[k] += ab;
    U.sys = slot;
  }
  std::vector<int> asys(L.n, slot);
  cudaStream_t st = B->st;
  Arena& A = B->A;
  prismq_status rc;
#define PQ_UP(dst, vec) \
  if ((rc = upload((dst), (vec), st)) != PRISMQ_OK) return rc;
  PQ_UP(A.pos + ab, L.pos);
  PQ_UP(A.vel + ab, L.vel);
  PQ_UP(A.xref + ab, L.pos);
  PQ_UP(A.lj + ab, L.lj);
  PQ_UP(A.atom_sys + ab, asys);
  PQ_UP(A.mask_all + ab, L.mask_all);
  PQ_UP(A.mask_ref + ab, L.mask_ref);
  PQ_UP(A.far + ab, L.far);
  PQ_UP(A.far_list + R.far_b, L.far_list);
  PQ_UP(A.inc + ab, L.inc);
  PQ_UP(A.inc_list + R.inc_b, L.inc_list);
  PQ_UP(A.ex_idx + ab, L.ex_idx);
  PQ_UP(A.ex_partner + R.ex_b, L.ex_partner);
  PQ_UP(A.ex_par + R.ex_b, L.ex_par);
  PQ_UP(A.bonds + R.bond_b, L.bonds);
  PQ_UP(A.angles + R.angle_b, L.angles);
  PQ_UP(A.dihs + R.dih_b, L.dihs);
  PQ_UP(A.units + R.unit_b, L.units);
  for (int k = 0; k < 4; ++k) R.units_by_nh[k] = 0;
  for (const Unit& u : L.units)
    if (u.nh >= 0 && u.nh <= 3) R.units_by_nh[3 - u.nh] += 1;
  PQ_UP(A.exc + R.exc_b, L.excs);
  PQ_UP(A.grp_refs + R.gref_b, L.grp_refs);
  PQ_UP(A.grp + ab / kForceGroup, L.grp);
#undef PQ_UP
  if (A.fp64) {
    std::vector<double4_32a> p64(L.n), v64(L.n);
    for (int a = 0; a < L.n; ++a) {
      p64[a] = make_double4_32a(L.pos[a].x, L.pos[a].y, L.pos[a].z, L.pos[a].w);
      v64[a] = make_double4_32a(L.vel[a].x, L.vel[a].y, L.vel[a].z, L.vel[a].w);
    }
    if ((rc = upload(A.pos64 + ab, p64, st)) != PRISMQ_OK) return rc;
    if ((rc = upload(A.vel64 + ab, v64, st)) != PRISMQ_OK) return rc;
    if ((rc = upload(A.lj64 + ab, L.lj64, st)) != PRISMQ_OK) return rc;
    for (int c = 0; c < 3; ++c) PQ_CK(cudaMemsetAsync(A.f64 + c * A.atom_cap + ab, 0, sizeof(double) * L.n, st));
    PQ_CK(cudaStreamSynchronize(st));  // the host staging vectors die here
  }
  PQ_CK(cudaMemsetAsync(A.nnbr + ab, 0, sizeof(int) * L.n, st));
  PQ_CK(cudaMemsetAsync(A.ntile + ab / 8, 0, sizeof(int) * ((L.n + 7) / 8), st));
  {
    // the atoms between the system's end and the next 32-atom boundary belong
    // to no system; tiles read them as the tail of the last j-cluster (with
    // no pair bit set), so they hold finite zeros
    const int64_t pad = ((ab + L.n + 31) / 32) * 32 - (ab + L.n);
    if (pad > 0) {
      PQ_CK(cudaMemsetAsync(A.pos + ab + L.n, 0, sizeof(float4) * pad, st));
      PQ_CK(cudaMemsetAsync(A.lj + ab + L.n, 0, sizeof(float2) * pad, st));
    }
  }
  PQ_CK(cudaMemsetAsync(A.f + ab, 0, sizeof(long long) * L.n, st));
  PQ_CK(cudaMemsetAsync(A.f + A.atom_cap + ab, 0, sizeof(long long) * L.n, st));
  PQ_CK(cudaMemsetAsync(A.f + 2 * A.atom_cap + ab, 0, sizeof(long long) * L.n, st));
  SysDev S;
  std::memset(&S, 0, sizeof(S));
  S.atom_begin = ab;
  S.n_atoms = L.n;
  S.unit_begin = (int)R.unit_b;
  S.n_units = (int)R.n_units;
  S.cell_begin = (int)R.cell_b;
  S.cell_cap = L.cell_cap;
  S.active = 1;
  S.nbr_mode = 0;
  fill_params(&S, p);
  for (int d = 0; d < 3; ++d) {
    S.ref_origin[d] = L.ref_origin[d];
    S.ref_dims[d] = L.ref_dims[d];
  }
  S.need_prime = 1;
  PQ_CK(cudaMemcpyAsync(A.sys + slot, &S, sizeof(S), cudaMemcpyHostToDevice, st));
  PQ_CK(cudaStreamSynchronize(st));
  R.active = true;
  R.ref_ok = L.ref_ok;
  R.need_prime = true;
  R.params = p;
  R.topo_hash = L.topo_hash;
  B->slots[slot] = R;
  B->h_sys[slot] = S;
  B->update_spans();
  if ((rc = B->upload_order()) != PRISMQ_OK) return rc;
  *slot_out = slot;
  return PRISMQ_OK;
}

prismq_status batch_release(prismq_batch* B, int slot) {
  if (slot < 0 || slot >= (int)B->slots.size() || !B->slots[slot].active)
    return fail(PRISMQ_E_NOT_FOUND, "no resident system in slot " + std::to_string(slot));
  SlotRec& R = B->slots[slot];
  Arena& A = B->A;
  cudaStream_t st = B->st;
  PQ_CK(cudaMemsetAsync(A.atom_sys + R.atom_b, 0xff, sizeof(int) * R.n_atoms, st));
  if (R.n_units)
    k_deactivate_units<<<(unsigned)((R.n_units + 255) / 256), 256, 0, st>>>(A.units + R.unit_b, R.n_units);
  PQ_CK(cudaMemsetAsync(A.grp + R.atom_b / kForceGroup, 0,
                        sizeof(int2) * ((R.n_atoms + kForceGroup - 1) / kForceGroup), st));
  PQ_CK(cudaMemsetAsync(A.sys + slot, 0, sizeof(SysDev), st));
  PQ_CK(cudaStreamSynchronize(st));
  if (R.fr_mem) cudaFree(R.fr_mem);
  B->r_atoms.release(R.atom_b, R.n_atoms);
  B->r_units.release(R.unit_b, R.n_units);
  B->r_bonds.release(R.bond_b, R.n_bonds);
  B->r_angles.release(R.angle_b, R.n_angles);
  B->r_dihs.release(R.dih_b, R.n_dihs);
  B->r_inc.release(R.inc_b, R.n_inc);
  B->r_ex.release(R.ex_b, R.n_ex);
  B->r_far.release(R.far_b, R.n_far);
  B->r_cells.release(R.cell_b, R.n_cell);
  B->r_exc.release(R.exc_b, R.n_exc);
  B->r_gref.release(R.gref_b, R.n_gref);
  R = SlotRec();
  B->update_spans();
  return B->upload_order();
}

prismq_status get_xyz(prismq_batch* B, int slot, float4* src_plane, float* out) {
  const SlotRec& R = B->slots[slot];
  const int n = (int)R.n_atoms;
  k_xyz_to_aos<<<(n + 255) / 256, 256, 0, B->st>>>(B->d_stage, src_plane + R.atom_b, n);
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaMemcpyAsync(out, B->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, B->st));
  PQ_CK(cudaStreamSynchronize(B->st));
  return PRISMQ_OK;
}

prismq_status set_xyz(prismq_batch* B, int slot, float4* dst_plane, const float* in) {
  const SlotRec& R = B->slots[slot];
  const int n = (int)R.n_atoms;
  for (int i = 0; i < 3 * n; ++i)
    if (!std::isfinite(in[i])) return fail(PRISMQ_E_INVALID, "non-finite input value");
  PQ_CK(cudaMemcpyAsync(B->d_stage, in, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, B->st));
  k_aos_to_xyz<<<(n + 255) / 256, 256, 0, B->st>>>(dst_plane + R.atom_b, B->d_stage, n);
  if (B->A.fp64) {  // the FP64 state takes the same values
    double4_32a* d64 = dst_plane == B->A.pos ? B->A.pos64 : B->A.vel64;
    k_aos_to_xyz64<<<(n + 255) / 256, 256, 0, B->st>>>(d64 + R.atom_b, B->d_stage, n);
  }
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaStreamSynchronize(B->st));
  return PRISMQ_OK;
}

prismq_status mark_prime(prismq_batch* B, int slot) {
  B->slots[slot].need_prime = true;
  const int one = 1;
  PQ_CK(cudaMemcpyAsync(&B->A.sys[slot].need_prime, &one, sizeof(int), cudaMemcpyHostToDevice, B->st));
  PQ_CK(cudaStreamSynchronize(B->st));
  return PRISMQ_OK;
}

prismq_status check_slot(prismq_batch* B, int slot) {
  if (!B) return fail(PRISMQ_E_INVALID, "batch is NULL");
  if (slot < 0 || slot >= (int)B->slots.size() || !B->slots[slot].active)
    return fail(PRISMQ_E_NOT_FOUND, "no resident system in slot " + std::to_string(slot));
  return PRISMQ_OK;
}

// Forces + per-atom energy planes at the current positions; returns the
// system's energy totals in out6 (host) when non-NULL.
prismq_status eval_energy(prismq_batch* B, int slot, double* out15) {
  prismq_status rc = B->prime_if_needed();
  if (rc != PRISMQ_OK) return rc;
  launch_force(B->A, B->atom_span, true, B->st, kSelAll, 0, B->group_slots);
  launch_energy_reduce(B->A, B->sys_span, B->d_energy, B->st);
  // the stepping kernels consume forces from the force-only variant
  launch_force(B->A, B->atom_span, false, B->st, kSelAll, 0, B->group_slots);
  g_launches += 3;
  PQ_CK(cudaGetLastError());
  if (out15) {
    PQ_CK(cudaMemcpyAsync(out15, B->d_energy + kEnergyOut * slot, sizeof(double) * kEnergyOut,
                          cudaMemcpyDeviceToHost, B->st));
  }
  PQ_CK(cudaStreamSynchronize(B->st));
  return B->check_status(slot);
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* prismq_last_error(void) { return g_err.c_str(); }
int prismq_abi_version(void) { return PRISMQ_ABI_VERSION; }
int prismq_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}
long long prismq_kernel_launches(void) { return g_launches.load(); }

prismq_status prismq_set_device(int32_t ordinal) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(PRISMQ_E_NO_DEVICE, "no CUDA device visible");
  }
  if (ordinal < 0 || ordinal >= n) return fail(PRISMQ_E_INVALID, "device ordinal out of range");
  const cudaError_t e = cudaSetDevice(ordinal);
  if (e != cudaSuccess) return fail(PRISMQ_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return PRISMQ_OK;
}

int32_t prismq_device_ordinal(void) {
  int n = 0, d = -1;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return d;
}

prismq_status prismq_device_info(int32_t out[3]) {
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  const int d = prismq_device_ordinal();
  if (d < 0) return fail(PRISMQ_E_NO_DEVICE, "no CUDA device visible");
  int sms = 0, khz = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d) != cudaSuccess ||
      cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, d) != cudaSuccess) {
    cudaGetLastError();
    return fail(PRISMQ_E_CUDA, "cudaDeviceGetAttribute failed");
  }
  out[0] = d;
  out[1] = sms;
  out[2] = khz;
  return PRISMQ_OK;
}

void prismq_params_default(prismq_params* p) {
  if (!p) return;
  p->dt = 0.004f;
  p->temperature = 300.0f;
  p->gamma = 1.0f;
  p->cutoff = 10.0f;
  p->skin = 2.0f;
  p->rebuild_interval = 20;
  p->com_interval = 100;
  p->max_constraint_iter = 100;
  p->seed = 0x50524953u;
  p->stream = 0u;
  p->shake_tol = 1.0e-4f;
  p->rattle_tol = 1.0e-5f;
  p->constraint_check_fp64 = 0;
  p->precision = PRISMQ_PRECISION_FP32;
}

void prismq_debug_noise(uint32_t seed, uint32_t stream, uint32_t atom, uint64_t step, uint32_t purpose,
                        float out3[3]) {
  normal3(seed, stream, atom, step, purpose, &out3[0], &out3[1], &out3[2]);
}

prismq_status prismq_polyala_build(int32_t n_chains, int32_t n_residues, uint64_t seed, float density,
                                   float box_edge, prismq_topology_buf** out) {
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  auto* b = new prismq_topology_buf();
  std::string err;
  if (!polyala_build(n_chains, n_residues, seed, density, box_edge, &b->topo, &err)) {
    delete b;
    return fail(PRISMQ_E_INVALID, err);
  }
  *out = b;
  return PRISMQ_OK;
}

prismq_status prismq_polyala_build_compact(int32_t n_chains, int32_t n_residues, uint64_t seed, float density,
                                           float box_edge, double* stats, prismq_topology_buf** out) {
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  auto* b = new prismq_topology_buf();
  std::string err;
  double st[4] = {0.0, 0.0, 0.0, 0.0};
  if (!polyala_build(n_chains, n_residues, seed, density, box_edge, &b->topo, &err, 1, st)) {
    delete b;
    return fail(PRISMQ_E_INVALID, err);
  }
  if (stats)
    for (int k = 0; k < 4; ++k) stats[k] = st[k];
  *out = b;
  return PRISMQ_OK;
}

prismq_status prismq_topology_view(const prismq_topology_buf* buf, prismq_topology* out) {
  if (!buf || !out) return fail(PRISMQ_E_INVALID, "NULL argument");
  buf->topo.view(out);
  return PRISMQ_OK;
}

void prismq_topology_free(prismq_topology_buf* buf) { delete buf; }

// ---- batch ----

prismq_status prismq_batch_create(int64_t max_atoms, int32_t max_systems, prismq_batch** out) {
  return prismq_batch_create_ex(max_atoms, max_systems, PRISMQ_PRECISION_FP32, out);
}

prismq_status prismq_batch_create_ex(int64_t max_atoms, int32_t max_systems, int32_t precision, prismq_batch** out) {
  if (!out || max_atoms <= 0 || max_systems <= 0) return fail(PRISMQ_E_INVALID, "invalid batch size");
  if (precision != PRISMQ_PRECISION_FP32 && precision != PRISMQ_PRECISION_FP64)
    return fail(PRISMQ_E_INVALID, "unknown precision");
  auto* B = new prismq_batch();
  prismq_status rc = batch_alloc_sized(B, max_atoms, max_systems, false, nullptr, precision);
  if (rc != PRISMQ_OK) {
    delete B;
    return rc;
  }
  *out = B;
  return PRISMQ_OK;
}

void prismq_batch_destroy(prismq_batch* b) { delete b; }

prismq_status prismq_batch_add_system(prismq_batch* b, const prismq_topology* topo,
                                      const prismq_params* params, int32_t* slot) {
  if (!b || !slot) return fail(PRISMQ_E_INVALID, "NULL argument");
  prismq_status rc = check_params(params);
  if (rc != PRISMQ_OK) return rc;
  Lowered L;
  rc = lower_topology(topo, &L);
  if (rc != PRISMQ_OK) return rc;
  init_velocities(&L, *params);
  int s = -1;
  rc = batch_admit(b, L, *params, &s);
  if (rc != PRISMQ_OK) return rc;
  *slot = s;
  return PRISMQ_OK;
}

prismq_status prismq_batch_remove_system(prismq_batch* b, int32_t slot) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  return batch_release(b, slot);
}

prismq_status prismq_batch_step(prismq_batch* b, int64_t n_steps) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  return b->step(n_steps);
}

prismq_status prismq_batch_get_state(prismq_batch* b, int32_t slot, float* xyz, float* vxyz) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (xyz && (rc = get_xyz(b, slot, b->A.pos, xyz)) != PRISMQ_OK) return rc;
  if (vxyz && (rc = get_xyz(b, slot, b->A.vel, vxyz)) != PRISMQ_OK) return rc;
  return PRISMQ_OK;
}

prismq_status prismq_batch_set_state(prismq_batch* b, int32_t slot, const float* xyz, const float* vxyz) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (xyz) {
    if ((rc = set_xyz(b, slot, b->A.pos, xyz)) != PRISMQ_OK) return rc;
    if ((rc = mark_prime(b, slot)) != PRISMQ_OK) return rc;
  }
  if (vxyz && (rc = set_xyz(b, slot, b->A.vel, vxyz)) != PRISMQ_OK) return rc;
  return PRISMQ_OK;
}

prismq_status prismq_batch_get_step(prismq_batch* b, int32_t slot, int64_t* step) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!step) return fail(PRISMQ_E_INVALID, "step is NULL");
  rc = b->sync_sys_from_device();
  if (rc != PRISMQ_OK) return rc;
  *step = b->h_sys[slot].step;
  return PRISMQ_OK;
}

prismq_status prismq_batch_set_force_variant(prismq_batch* b, int32_t variant, int32_t* n_variants) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  if (n_variants) *n_variants = force_variant_count();
  if (variant < -1 || variant >= force_variant_count()) return fail(PRISMQ_E_INVALID, "no such force variant");
  if (variant != b->force_variant) b->graph_dirty = true;
  b->force_pinned = variant >= 0;
  b->force_variant = variant;
  b->tuned_span = 0;
  return PRISMQ_OK;
}

prismq_status prismq_batch_set_pair_layout(prismq_batch* b, int32_t layout) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  if (layout != 0 && layout != 1) return fail(PRISMQ_E_INVALID, "pair layout must be 0 (rows) or 1 (tiles)");
  if (layout == b->A.pair_layout) return PRISMQ_OK;
  b->A.pair_layout = layout;
  b->graph_dirty = true;
  for (int s = 0; s < (int)b->slots.size(); ++s) {
    if (!b->slots[s].active) continue;
    const prismq_status rc = mark_prime(b, s);
    if (rc != PRISMQ_OK) return rc;
  }
  return PRISMQ_OK;
}

int32_t prismq_batch_pair_layout(const prismq_batch* b) { return b ? b->A.pair_layout : -1; }

prismq_status prismq_set_pair_layout(prismq_system* sys, int32_t layout) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_set_pair_layout(sys->b, layout);
}

prismq_status prismq_batch_tuning_ex(prismq_batch* b, int32_t out[5]) {
  if (!b || !out) return fail(PRISMQ_E_INVALID, "NULL argument");
  out[0] = b->force_variant;
  out[1] = out[2] = out[3] = out[4] = 0;
  if (b->force_variant >= 0) {
    force_variant_shape(b->force_variant, &out[1], &out[2]);
    out[3] = out[1] / kLanes;
    out[4] = force_variant_prefetch(b->force_variant);
  }
  return PRISMQ_OK;
}

prismq_status prismq_batch_tuning(prismq_batch* b, int32_t out[3]) {
  if (!b || !out) return fail(PRISMQ_E_INVALID, "NULL argument");
  out[0] = b->force_variant;
  out[1] = out[2] = 0;
  if (b->force_variant >= 0) force_variant_shape(b->force_variant, &out[1], &out[2]);
  return PRISMQ_OK;
}

prismq_status prismq_batch_counters(prismq_batch* b, int32_t slot, int64_t out[2]) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  rc = b->sync_sys_from_device();
  if (rc != PRISMQ_OK) return rc;
  out[0] = b->h_sys[slot].step;
  out[1] = b->h_sys[slot].n_rebuilds;
  return PRISMQ_OK;
}

prismq_status prismq_batch_status(prismq_batch* b, int32_t slot) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  return b->check_status(slot);
}

prismq_status prismq_batch_virial(prismq_batch* b, int32_t slot, double out[9]) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  double e[kEnergyOut];
  rc = eval_energy(b, slot, e);
  if (rc != PRISMQ_OK) return rc;
  for (int i = 0; i < 9; ++i) out[i] = e[6 + i];
  return PRISMQ_OK;
}

prismq_status prismq_batch_get_state_f64(prismq_batch* b, int32_t slot, double* xyz, double* vxyz) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  const SlotRec& R = b->slots[slot];
  const int n = (int)R.n_atoms;
  if (!b->d_stage64) PQ_CK(cudaMalloc((void**)&b->d_stage64, sizeof(double) * 3 * b->A.atom_cap));
  for (int w = 0; w < 2; ++w) {
    double* out = w == 0 ? xyz : vxyz;
    if (!out) continue;
    if (b->A.fp64)
      k_xyz64_to_aos<<<(n + 255) / 256, 256, 0, b->st>>>(b->d_stage64, (w == 0 ? b->A.pos64 : b->A.vel64) + R.atom_b, n);
    else
      k_xyz_to_aos64<<<(n + 255) / 256, 256, 0, b->st>>>(b->d_stage64, (w == 0 ? b->A.pos : b->A.vel) + R.atom_b, n);
    PQ_CK(cudaGetLastError());
    PQ_CK(cudaMemcpyAsync(out, b->d_stage64, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, b->st));
    PQ_CK(cudaStreamSynchronize(b->st));
  }
  return PRISMQ_OK;
}

prismq_status prismq_batch_get_forces_f64(prismq_batch* b, int32_t slot, double* f) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!f) return fail(PRISMQ_E_INVALID, "f is NULL");
  const SlotRec& R = b->slots[slot];
  const int64_t n = R.n_atoms;
  if (b->A.fp64) {
    std::vector<double> h(3 * n);
    for (int c = 0; c < 3; ++c)
      PQ_CK(cudaMemcpyAsync(h.data() + c * n, b->A.f64 + c * b->A.atom_cap + R.atom_b, sizeof(double) * n,
                            cudaMemcpyDeviceToHost, b->st));
    PQ_CK(cudaStreamSynchronize(b->st));
    for (int64_t a = 0; a < n; ++a)
      for (int c = 0; c < 3; ++c) f[3 * a + c] = h[c * n + a];
  } else {
    std::vector<long long> h(3 * n);
    for (int c = 0; c < 3; ++c)
      PQ_CK(cudaMemcpyAsync(h.data() + c * n, b->A.f + c * b->A.atom_cap + R.atom_b, sizeof(long long) * n,
                            cudaMemcpyDeviceToHost, b->st));
    PQ_CK(cudaStreamSynchronize(b->st));
    for (int64_t a = 0; a < n; ++a)
      for (int c = 0; c < 3; ++c) f[3 * a + c] = (double)h[c * n + a] * kFixedInvD;
  }
  return PRISMQ_OK;
}

prismq_status prismq_batch_energy(prismq_batch* b, int32_t slot, double out[6]) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  double e[kEnergyOut];
  rc = eval_energy(b, slot, e);
  if (rc != PRISMQ_OK) return rc;
  // five potential planes in order: bond, angle, dihedral, exception, nonbonded; then kinetic
  for (int i = 0; i < 6; ++i) out[i] = e[i];
  return PRISMQ_OK;
}

prismq_status prismq_batch_run_timed(prismq_batch* b, int64_t n_steps, float* total_ms, float* phase_ms) {
  if (!b || !total_ms) return fail(PRISMQ_E_INVALID, "NULL argument");
  return b->run_timed(n_steps, total_ms, phase_ms);
}

prismq_status prismq_batch_time_force(prismq_batch* b, int32_t n_launches, float* ms_per_launch) {
  if (!b || !ms_per_launch) return fail(PRISMQ_E_INVALID, "NULL argument");
  return b->time_force(n_launches, ms_per_launch);
}

int64_t prismq_batch_atom_span(const prismq_batch* b) { return b ? b->atom_span : 0; }

int64_t prismq_batch_atom_offset(const prismq_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return -1;
  return b->slots[slot].atom_b;
}

// Host arrays in pinned memory are read (written) by the transfer kernel
// directly; pageable ones go through the device staging buffers.
prismq_status prismq_batch_set_state_all(prismq_batch* b, const float* xyz, const float* vxyz) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  const int64_t n = b->atom_span;
  if (n == 0) return PRISMQ_OK;
  const float* xs = mapped_host(xyz);
  const float* vs = mapped_host(vxyz);
  if (xyz && !xs) {
    PQ_CK(cudaMemcpyAsync(b->d_stage, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, b->st));
    xs = b->d_stage;
  }
  if (vxyz && !vs) {
    PQ_CK(cudaMemcpyAsync(b->d_stage2, vxyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, b->st));
    vs = b->d_stage2;
  }
  const int vec = (!xs || aligned16(xs)) && (!vs || aligned16(vs));
  k_set_state_all<<<(unsigned)((n + kStateBlock - 1) / kStateBlock), kStateBlock, 0, b->st>>>(
      b->A.pos, b->A.vel, b->A.pos64, b->A.vel64, xs, vs, b->A.atom_sys, b->A.sys, n, vec);
  g_launches += 1;
  PQ_CK(cudaGetLastError());
  if (xyz) return b->prime_flagged();
  return PRISMQ_OK;
}

// Enqueue the whole-arena read-back on the batch stream (no synchronisation).
static prismq_status enqueue_get_state_all(prismq_batch* b, float* xyz, float* vxyz) {
  const int64_t n = b->atom_span;
  if (n == 0) return PRISMQ_OK;
  float* xd = const_cast<float*>(mapped_host(xyz));
  float* vd = const_cast<float*>(mapped_host(vxyz));
  const bool stage_x = xyz && !xd, stage_v = vxyz && !vd;
  if (stage_x) xd = b->d_stage;
  if (stage_v) vd = b->d_stage2;
  const int vec = (!xd || aligned16(xd)) && (!vd || aligned16(vd));
  k_get_state_all<<<(unsigned)((n + kStateBlock - 1) / kStateBlock), kStateBlock, 0, b->st>>>(b->A.pos, b->A.vel,
                                                                                            xd, vd, n, vec);
  g_launches += 1;
  PQ_CK(cudaGetLastError());
  if (stage_x) PQ_CK(cudaMemcpyAsync(xyz, b->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->st));
  if (stage_v) PQ_CK(cudaMemcpyAsync(vxyz, b->d_stage2, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->st));
  return PRISMQ_OK;
}

prismq_status prismq_batch_get_state_all(prismq_batch* b, float* xyz, float* vxyz) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  prismq_status rc = enqueue_get_state_all(b, xyz, vxyz);
  if (rc != PRISMQ_OK) return rc;
  PQ_CK(cudaStreamSynchronize(b->st));
  return PRISMQ_OK;
}

// Upload, n steps and read-back in one call: the three are enqueued back to
// back and the host waits once, for the state and the status words together.
prismq_status prismq_batch_step_host(prismq_batch* b, int64_t n_steps, const float* xyz_in, const float* vxyz_in,
                                     float* xyz_out, float* vxyz_out) {
  if (!b) return fail(PRISMQ_E_INVALID, "batch is NULL");
  prismq_status rc = prismq_batch_set_state_all(b, xyz_in, vxyz_in);
  if (rc != PRISMQ_OK) return rc;
  prismq_status step_rc = PRISMQ_OK;
  bool status_pending = false;  // the steps' status words are read after the state
  if (n_steps > 0 && b->sys_span > 0) {
    if (b->recording_frames()) {
      step_rc = b->step(n_steps);  // frame segments synchronise on their own
    } else {
      if ((rc = b->step_segment(n_steps, false)) != PRISMQ_OK) return rc;
      status_pending = true;
    }
  }
  if (status_pending && xyz_out && mapped_host(xyz_out)) {
    // positions on st3 from the tail graph's ev_xready on (packed on the
    // device, then one DMA copy into the pinned array, beside the last step's
    // forces), velocities on st after the tail; st then waits for st3
    const int64_t n = b->atom_span;
    const unsigned blocks = (unsigned)((n + kStateBlock - 1) / kStateBlock);
    PQ_CK(cudaStreamWaitEvent(b->st3, b->ev_xready, 0));
    k_get_state_all<<<blocks, kStateBlock, 0, b->st3>>>(b->A.pos, b->A.vel, b->d_stage, nullptr, n, 1);
    PQ_CK(cudaMemcpyAsync(xyz_out, b->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->st3));
    PQ_CK(cudaEventRecord(b->ev_xdone, b->st3));
    g_launches += 1;
    if ((rc = enqueue_get_state_all(b, nullptr, vxyz_out)) != PRISMQ_OK) return rc;
    PQ_CK(cudaStreamWaitEvent(b->st, b->ev_xdone, 0));
    PQ_CK(cudaGetLastError());
  } else if ((rc = enqueue_get_state_all(b, xyz_out, vxyz_out)) != PRISMQ_OK) {
    return rc;
  }
  if (status_pending) return b->check_status();  // its read-back waits for the state too
  PQ_CK(cudaStreamSynchronize(b->st));
  return step_rc;
}

int64_t prismq_batch_resident_atoms(const prismq_batch* b) {
  if (!b) return 0;
  int64_t n = 0;
  for (auto& s : b->slots)
    if (s.active) n += s.n_atoms;
  return n;
}

int32_t prismq_batch_resident_systems(const prismq_batch* b) {
  if (!b) return 0;
  int32_t n = 0;
  for (auto& s : b->slots)
    if (s.active) ++n;
  return n;
}

// ---- single system ----

prismq_status prismq_system_create(const prismq_topology* topo, const prismq_params* params,
                                   prismq_system** out) {
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  prismq_status rc = check_params(params);
  if (rc != PRISMQ_OK) return rc;
  Lowered L;
  rc = lower_topology(topo, &L);
  if (rc != PRISMQ_OK) return rc;
  init_velocities(&L, *params);
  auto* B = new prismq_batch();
  const int64_t n = L.n;
  rc = batch_alloc(B, n, 1, (int64_t)L.bonds.size(), (int64_t)L.angles.size(), (int64_t)L.dihs.size(),
                   (int64_t)L.inc_list.size(), (int64_t)L.ex_partner.size(), (int64_t)L.far_list.size(),
                   2 * ((int64_t)L.cell_cap + 1), (int64_t)L.excs.size(), (int64_t)L.grp_refs.size(),
                   params->precision);
  if (rc != PRISMQ_OK) {
    delete B;
    return rc;
  }
  int slot = -1;
  rc = batch_admit(B, L, *params, &slot);
  if (rc != PRISMQ_OK) {
    delete B;
    return rc;
  }
  auto* s = new prismq_system();
  s->b = B;
  s->slot = slot;
  *out = s;
  return PRISMQ_OK;
}

void prismq_system_destroy(prismq_system* sys) {
  if (!sys) return;
  delete sys->b;
  delete sys;
}

int32_t prismq_system_n_atoms(const prismq_system* sys) {
  return sys ? (int32_t)sys->b->slots[sys->slot].n_atoms : 0;
}

static prismq_status set_param_field(prismq_system* sys, int which, float v) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  prismq_params p = sys->b->slots[sys->slot].params;
  if (which == 0) p.dt = v;
  if (which == 1) p.temperature = v;
  if (which == 2) p.gamma = v;
  prismq_status rc = check_params(&p);
  if (rc != PRISMQ_OK) return rc;
  prismq_batch* B = sys->b;
  rc = B->sync_sys_from_device();
  if (rc != PRISMQ_OK) return rc;
  SysDev S = B->h_sys[sys->slot];
  if (S.proto.on) {
    // a protocol owns T and γ; set_dt moves its base timestep (fused_engine.rs:15342)
    if (which != 0) return fail(PRISMQ_E_INVALID, "a run protocol controls temperature and friction; remove it first");
    S.proto.base_dt = v;
    protocol_now(&S);
  } else {
    fill_params(&S, p);
  }
  PQ_CK(cudaMemcpyAsync(B->A.sys + sys->slot, &S, sizeof(S), cudaMemcpyHostToDevice, B->st));
  PQ_CK(cudaStreamSynchronize(B->st));
  B->h_sys[sys->slot] = S;
  B->slots[sys->slot].params = p;
  return PRISMQ_OK;
}

prismq_status prismq_set_dt(prismq_system* sys, float dt) { return set_param_field(sys, 0, dt); }
prismq_status prismq_set_temperature(prismq_system* sys, float t) { return set_param_field(sys, 1, t); }
prismq_status prismq_set_gamma(prismq_system* sys, float g) { return set_param_field(sys, 2, g); }

prismq_status prismq_set_positions(prismq_system* sys, const float* xyz) {
  if (!sys || !xyz) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_set_state(sys->b, sys->slot, xyz, nullptr);
}
prismq_status prismq_set_velocities(prismq_system* sys, const float* vxyz) {
  if (!sys || !vxyz) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_set_state(sys->b, sys->slot, nullptr, vxyz);
}
prismq_status prismq_get_positions(prismq_system* sys, float* xyz) {
  if (!sys || !xyz) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_get_state(sys->b, sys->slot, xyz, nullptr);
}
prismq_status prismq_get_velocities(prismq_system* sys, float* vxyz) {
  if (!sys || !vxyz) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_get_state(sys->b, sys->slot, nullptr, vxyz);
}
prismq_status prismq_get_step(prismq_system* sys, int64_t* step) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_get_step(sys->b, sys->slot, step);
}
prismq_status prismq_set_step(prismq_system* sys, int64_t step) {
  if (!sys || step < 0) return fail(PRISMQ_E_INVALID, "invalid argument");
  prismq_batch* B = sys->b;
  prismq_status rc = B->sync_sys_from_device();
  if (rc != PRISMQ_OK) return rc;
  SysDev S = B->h_sys[sys->slot];
  S.step = step;
  protocol_now(&S);  // the next step's parameters follow the counter
  PQ_CK(cudaMemcpyAsync(B->A.sys + sys->slot, &S, sizeof(S), cudaMemcpyHostToDevice, B->st));
  PQ_CK(cudaStreamSynchronize(B->st));
  B->h_sys[sys->slot] = S;
  return PRISMQ_OK;
}

void prismq_protocol_default(prismq_protocol* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->start_temp = 300.0f;
  p->end_temp = 300.0f;
  p->warm_hold_steps = 100000;  // TemperatureProtocol::physiological (fused_engine.rs:2996-3004)
  p->gamma_base = 1.0f;
  p->equilibration_steps = 10000;  // ProtocolState::from_cryo_uv (protocol_state.rs:676-677)
  p->equilibration_gamma = 1000.0f;
  p->base_dt = 0.004f;
}

prismq_status prismq_protocol_eval(const prismq_protocol* p, int64_t director_step, float out[3]) {
  prismq_status rc = check_protocol(p);
  if (rc != PRISMQ_OK) return rc;
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  StepParams P;
  protocol_eval(protocol_dev(*p, 0), director_step, &P);
  out[0] = P.temperature;
  out[1] = P.gamma;
  out[2] = P.dt;
  return PRISMQ_OK;
}

prismq_status prismq_batch_set_protocol(prismq_batch* b, int32_t slot, const prismq_protocol* p) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (p && (rc = check_protocol(p)) != PRISMQ_OK) return rc;
  if ((rc = b->sync_sys_from_device()) != PRISMQ_OK) return rc;
  SysDev S = b->h_sys[slot];
  if (p) {
    // the next step is director step current_step + 1
    S.proto = protocol_dev(*p, S.step - ((long long)p->current_step + 1));
    protocol_now(&S);
  } else {
    S.proto.on = 0;
    carry_post(&S);
    prismq_params& q = b->slots[slot].params;
    q.dt = S.dt;
    q.temperature = S.temperature;
    q.gamma = S.gamma;
  }
  PQ_CK(cudaMemcpyAsync(b->A.sys + slot, &S, sizeof(S), cudaMemcpyHostToDevice, b->st));
  PQ_CK(cudaStreamSynchronize(b->st));
  b->h_sys[slot] = S;
  return PRISMQ_OK;
}

prismq_status prismq_batch_get_step_params(prismq_batch* b, int32_t slot, float out[3]) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!out) return fail(PRISMQ_E_INVALID, "out is NULL");
  if ((rc = b->sync_sys_from_device()) != PRISMQ_OK) return rc;
  const SysDev& S = b->h_sys[slot];
  out[0] = S.temperature;
  out[1] = S.gamma;
  out[2] = S.dt;
  return PRISMQ_OK;
}

prismq_status prismq_set_protocol(prismq_system* sys, const prismq_protocol* p) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_set_protocol(sys->b, sys->slot, p);
}

prismq_status prismq_get_step_params(prismq_system* sys, float out[3]) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_get_step_params(sys->b, sys->slot, out);
}

prismq_status prismq_step(prismq_system* sys, int64_t n_steps) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  if (n_steps < 0) return fail(PRISMQ_E_INVALID, "n_steps must be >= 0");
  return sys->b->step(n_steps);
}

prismq_status prismq_compute_forces(prismq_system* sys, double* pe_total, float* f_aos, int64_t* f_fixed) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  prismq_batch* B = sys->b;
  double e[kEnergyOut];
  prismq_status rc = eval_energy(B, sys->slot, e);
  if (rc != PRISMQ_OK) return rc;
  if (pe_total) *pe_total = e[0] + e[1] + e[2] + e[3] + e[4];
  if ((f_aos || f_fixed) && B->A.fp64) {
    const int64_t n = B->slots[sys->slot].n_atoms;
    std::vector<double> h(3 * n);
    if ((rc = prismq_batch_get_forces_f64(B, sys->slot, h.data())) != PRISMQ_OK) return rc;
    for (int64_t i = 0; i < 3 * n; ++i) {
      if (f_aos) f_aos[i] = (float)h[i];
      if (f_fixed) {
        const double v = h[i] * 4294967296.0;
        f_fixed[i] = !(v == v) ? 0 : v >= 9.2233720368547758e18 ? INT64_MAX : v <= -9.2233720368547758e18 ? INT64_MIN : (int64_t)std::llrint(v);
      }
    }
  } else if (f_aos || f_fixed) {
    const SlotRec& R = B->slots[sys->slot];
    const int64_t n = R.n_atoms;
    std::vector<long long> h(3 * n);
    for (int c = 0; c < 3; ++c)
      PQ_CK(cudaMemcpyAsync(h.data() + c * n, B->A.f + c * B->A.atom_cap + R.atom_b, sizeof(long long) * n,
                            cudaMemcpyDeviceToHost, B->st));
    PQ_CK(cudaStreamSynchronize(B->st));
    for (int64_t a = 0; a < n; ++a)
      for (int c = 0; c < 3; ++c) {
        const long long v = h[c * n + a];
        if (f_fixed) f_fixed[3 * a + c] = v;
        if (f_aos) f_aos[3 * a + c] = fixed2f(v);
      }
  }
  return PRISMQ_OK;
}

prismq_status prismq_energy_components(prismq_system* sys, double out[6]) {
  if (!sys || !out) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_energy(sys->b, sys->slot, out);
}

prismq_status prismq_virial(prismq_system* sys, double out[9]) {
  if (!sys || !out) return fail(PRISMQ_E_INVALID, "NULL argument");
  return prismq_batch_virial(sys->b, sys->slot, out);
}

prismq_status prismq_get_state_f64(prismq_system* sys, double* xyz, double* vxyz) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_get_state_f64(sys->b, sys->slot, xyz, vxyz);
}

prismq_status prismq_get_forces_f64(prismq_system* sys, double* f) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_get_forces_f64(sys->b, sys->slot, f);
}

prismq_status prismq_build_neighbors(prismq_system* sys, prismq_nlist_mode mode, int32_t* pairs_out, size_t cap,
                                     size_t* n_out) {
  if (!sys || !n_out) return fail(PRISMQ_E_INVALID, "NULL argument");
  if (mode != PRISMQ_NLIST_COMPLETE && mode != PRISMQ_NLIST_REF27) return fail(PRISMQ_E_INVALID, "unknown mode");
  prismq_batch* B = sys->b;
  const SlotRec& R = B->slots[sys->slot];
  if (mode == PRISMQ_NLIST_REF27 && !R.ref_ok)
    return fail(PRISMQ_E_INVALID, "reference grid needs more than 32 cells per axis for this system");
  B->control(kCtlForce, (int)mode, B->st);
  launch_nbr_build(B->A, B->atom_span, 0, B->st);
  launch_force(B->A, B->atom_span, false, B->st, kSelAll, 0, B->group_slots);  // also clears the rebuild queue
  g_launches += 3 + (B->max_big_atoms > 0 ? 4 : 0);
  PQ_CK(cudaGetLastError());
  const int64_t n = R.n_atoms, ab = R.atom_b;
  const int64_t g0 = ab / 8, g1 = (ab + n + 7) / 8;
  SysDev probe{};
  probe.nbr_mode = mode == PRISMQ_NLIST_REF27 ? 1 : 0;
  const bool tiles = uses_tiles(B->A, probe);
  std::vector<int> cnt, rows, ntile;
  std::vector<int2> tl;
  if (tiles) {
    ntile.resize(g1 - g0);
    tl.resize((size_t)(g1 - g0) * kTileCap);
    PQ_CK(cudaMemcpyAsync(ntile.data(), B->A.ntile + g0, sizeof(int) * ntile.size(), cudaMemcpyDeviceToHost,
                          B->st));
    PQ_CK(cudaMemcpyAsync(tl.data(), B->A.tiles + g0 * kTileCap, sizeof(int2) * tl.size(), cudaMemcpyDeviceToHost,
                          B->st));
  } else {
    cnt.resize(n);
    rows.resize((size_t)(g1 - g0) * kNbrCap * 8);
    PQ_CK(cudaMemcpyAsync(cnt.data(), B->A.nnbr + ab, sizeof(int) * n, cudaMemcpyDeviceToHost, B->st));
    PQ_CK(cudaMemcpyAsync(rows.data(), B->A.nbr + g0 * kNbrCap * 8, sizeof(int) * rows.size(),
                          cudaMemcpyDeviceToHost, B->st));
  }
  PQ_CK(cudaStreamSynchronize(B->st));
  prismq_status st = B->check_status(sys->slot);
  // restore the production list
  B->control(kCtlForce, 0, B->st);
  launch_nbr_build(B->A, B->atom_span, 1, B->st);
  launch_force(B->A, B->atom_span, false, B->st, kSelAll, 0, B->group_slots);
  g_launches += 3 + (B->max_big_atoms > 0 ? 4 : 0);
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaStreamSynchronize(B->st));
  if (st != PRISMQ_OK) return st;
  std::vector<std::pair<int, int>> pairs;
  if (tiles) {
    // every set bit of a tile is one pair of the list (both orders appear)
    for (int64_t g = g0; g < g1; ++g)
      for (int t = 0; t < ntile[g - g0]; ++t) {
        const int2 e = tl[(size_t)(g - g0) * kTileCap + t];
        for (int bit = 0; bit < 32; ++bit) {
          if (!(((unsigned)e.y >> bit) & 1u)) continue;
          const int i = (int)(8 * g + (bit & 7) - ab), j = 4 * e.x + (bit >> 3) - (int)ab;
          if (j > i) pairs.emplace_back(i, j);
        }
      }
  } else {
    for (int64_t i = 0; i < n; ++i) {
      const int64_t a = ab + i;
      for (int k = 0; k < cnt[i]; ++k) {
        const int j = rows[nbr_index(a, k) - g0 * kNbrCap * 8] - (int)ab;
        if (j > i) pairs.emplace_back((int)i, j);
      }
    }
  }
  std::sort(pairs.begin(), pairs.end());
  *n_out = pairs.size();
  if (pairs.size() > cap || (!pairs_out && !pairs.empty()))
    return fail(PRISMQ_E_CAPACITY, "pairs_out holds fewer than the pairs found");
  for (size_t q = 0; q < pairs.size(); ++q) {
    pairs_out[2 * q] = pairs[q].first;
    pairs_out[2 * q + 1] = pairs[q].second;
  }
  return PRISMQ_OK;
}

prismq_status prismq_debug_phases(prismq_system* sys, prismq_phase_set set, int64_t step) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  if (set != PRISMQ_PHASES_PRE && set != PRISMQ_PHASES_POST) return fail(PRISMQ_E_INVALID, "unknown phase set");
  prismq_batch* B = sys->b;
  if (B->A.fp64) return fail(PRISMQ_E_INVALID, "single phase sets are an FP32 parity entry point");
  prismq_status rc = B->prime_if_needed();
  if (rc != PRISMQ_OK) return rc;
  launch_debug_phases(B->A, B->unit_span, set == PRISMQ_PHASES_PRE ? kIntPre : kIntPost, step, B->st);
  g_launches += 1;
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaStreamSynchronize(B->st));
  return B->check_status(sys->slot);
}

// ---------------------------------------------------------------------------
// Checkpoints: the complete dynamic state of one system at a step boundary.
// A restored system continues bit for bit as if it had never stopped.  The
// noise is counter-based (no generator state) and the forces are recomputed
// from the saved positions over neighbour rows rebuilt from the saved
// list-build positions, which reproduces the rows, their order and so the
// forces exactly.
// ---------------------------------------------------------------------------
namespace {

struct CkptHeader {
  char magic[8];          // "PQCKPT" 0 1
  uint32_t version;       // 1
  uint32_t header_bytes;  // sizeof(CkptHeader)
  int32_t n_atoms, precision;
  uint64_t topo_hash;
  int64_t step, n_rebuilds;
  int32_t steps_since_rebuild, built, displaced, nbr_mode;
  int32_t pending_prime, pad0;
  prismq_params params;
  float dt, temperature, gamma, c1;
  double c1d;
  ProtocolDev proto;
  float ref_origin[3];
  int32_t ref_dims[3];
  uint64_t payload_bytes;
  uint64_t payload_hash;  // x, v and list-build positions, float AoS
};
constexpr char kCkptMagic[8] = {'P', 'Q', 'C', 'K', 'P', 'T', 0, 1};

size_t ckpt_bytes(int64_t n) { return sizeof(CkptHeader) + 3 * 3 * sizeof(float) * (size_t)n; }

}  // namespace

prismq_status prismq_batch_checkpoint_size(prismq_batch* b, int32_t slot, size_t* bytes) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!bytes) return fail(PRISMQ_E_INVALID, "bytes is NULL");
  *bytes = ckpt_bytes(b->slots[slot].n_atoms);
  return PRISMQ_OK;
}

prismq_status prismq_batch_checkpoint_save(prismq_batch* b, int32_t slot, void* buf, size_t cap, size_t* written) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!buf) return fail(PRISMQ_E_INVALID, "buffer is NULL");
  if (b->A.fp64) return fail(PRISMQ_E_INVALID, "checkpoints cover FP32 systems");
  const SlotRec& R = b->slots[slot];
  const int64_t n = R.n_atoms;
  if (cap < ckpt_bytes(n)) return fail(PRISMQ_E_CAPACITY, "checkpoint buffer too small");
  if ((rc = b->check_status(slot)) != PRISMQ_OK) return rc;  // a failed system has no state to resume
  const SysDev& S = b->h_sys[slot];
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.header_bytes = sizeof(CkptHeader);
  h.n_atoms = (int32_t)n;
  h.precision = PRISMQ_PRECISION_FP32;
  h.topo_hash = R.topo_hash;
  h.step = S.step;
  h.n_rebuilds = S.n_rebuilds;
  h.steps_since_rebuild = S.steps_since_rebuild;
  h.built = S.built;
  h.displaced = S.displaced;
  h.nbr_mode = S.nbr_mode;
  h.pending_prime = (R.need_prime || S.need_prime || !S.built) ? 1 : 0;
  h.params = R.params;
  h.dt = S.dt;
  h.temperature = S.temperature;
  h.gamma = S.gamma;
  h.c1 = S.c1;
  h.c1d = S.c1d;
  h.proto = S.proto;
  for (int d = 0; d < 3; ++d) {
    h.ref_origin[d] = S.ref_origin[d];
    h.ref_dims[d] = S.ref_dims[d];
  }
  h.payload_bytes = 9 * sizeof(float) * (size_t)n;
  float* x = reinterpret_cast<float*>(static_cast<char*>(buf) + sizeof(CkptHeader));
  if ((rc = get_xyz(b, slot, b->A.pos, x)) != PRISMQ_OK) return rc;
  if ((rc = get_xyz(b, slot, b->A.vel, x + 3 * n)) != PRISMQ_OK) return rc;
  if ((rc = get_xyz(b, slot, b->A.xref, x + 6 * n)) != PRISMQ_OK) return rc;
  h.payload_hash = fnv_words(14695981039346656037ull, x, h.payload_bytes);
  std::memcpy(buf, &h, sizeof(h));
  if (written) *written = ckpt_bytes(n);
  return PRISMQ_OK;
}

prismq_status prismq_batch_checkpoint_restore(prismq_batch* b, int32_t slot, const void* buf, size_t len) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!buf) return fail(PRISMQ_E_INVALID, "buffer is NULL");
  if (b->A.fp64) return fail(PRISMQ_E_INVALID, "checkpoints cover FP32 systems");
  SlotRec& R = b->slots[slot];
  const int64_t n = R.n_atoms;
  CkptHeader h;
  if (len < sizeof(h)) return fail(PRISMQ_E_INVALID, "checkpoint truncated");
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1 || h.header_bytes != sizeof(CkptHeader))
    return fail(PRISMQ_E_INVALID, "not a checkpoint of this library version");
  if (h.n_atoms != n || h.precision != PRISMQ_PRECISION_FP32)
    return fail(PRISMQ_E_INVALID, "checkpoint is for a system of another size or precision");
  if (h.topo_hash != R.topo_hash) return fail(PRISMQ_E_INVALID, "checkpoint belongs to another topology");
  if (h.payload_bytes != 9 * sizeof(float) * (size_t)n || len != ckpt_bytes(n))
    return fail(PRISMQ_E_INVALID, "checkpoint truncated or padded");
  const float* x = reinterpret_cast<const float*>(static_cast<const char*>(buf) + sizeof(CkptHeader));
  if (fnv_words(14695981039346656037ull, x, h.payload_bytes) != h.payload_hash)
    return fail(PRISMQ_E_INVALID, "checkpoint payload is corrupted");
  if ((rc = check_params(&h.params)) != PRISMQ_OK) return rc;
  if (h.params.precision != PRISMQ_PRECISION_FP32) return fail(PRISMQ_E_INVALID, "checkpoint precision");
  if (h.step < 0 || h.built < 0 || h.built > 1 || (h.nbr_mode != 0 && h.nbr_mode != 1))
    return fail(PRISMQ_E_INVALID, "checkpoint control state out of range");
  if ((rc = b->sync_sys_from_device()) != PRISMQ_OK) return rc;
  SysDev S = b->h_sys[slot];
  S.status = 0;
  S.nbr_mode = h.nbr_mode;
  for (int d = 0; d < 3; ++d) {
    S.ref_origin[d] = h.ref_origin[d];
    S.ref_dims[d] = h.ref_dims[d];
  }
  fill_params(&S, h.params);
  if (!h.pending_prime) {
    // rebuild the rows from the positions of the last list build, then
    // evaluate the forces at the saved positions over them
    if ((rc = set_xyz(b, slot, b->A.pos, x + 6 * n)) != PRISMQ_OK) return rc;
    S.need_prime = 1;
    S.built = 0;
    PQ_CK(cudaMemcpyAsync(b->A.sys + slot, &S, sizeof(S), cudaMemcpyHostToDevice, b->st));
    if ((rc = b->prime_flagged()) != PRISMQ_OK) return rc;
    if ((rc = set_xyz(b, slot, b->A.pos, x)) != PRISMQ_OK) return rc;
    launch_force(b->A, b->atom_span, false, b->st, kSelRebuilding, 0, b->group_slots);
    g_launches += 1;
    PQ_CK(cudaGetLastError());
    if ((rc = b->sync_sys_from_device()) != PRISMQ_OK) return rc;
    S = b->h_sys[slot];
    if (S.status != 0) return b->check_status(slot);
  } else if ((rc = set_xyz(b, slot, b->A.pos, x)) != PRISMQ_OK) {
    return rc;
  }
  if ((rc = set_xyz(b, slot, b->A.vel, x + 3 * n)) != PRISMQ_OK) return rc;
  S.step = h.step;
  S.n_rebuilds = h.n_rebuilds;
  S.steps_since_rebuild = h.steps_since_rebuild;
  S.built = h.built;
  S.displaced = h.displaced;
  S.need_prime = h.pending_prime;
  S.dt = h.dt;
  S.temperature = h.temperature;
  S.gamma = h.gamma;
  S.c1 = h.c1;
  S.c1d = h.c1d;
  carry_post(&S);
  S.proto = h.proto;
  PQ_CK(cudaMemcpyAsync(b->A.sys + slot, &S, sizeof(S), cudaMemcpyHostToDevice, b->st));
  PQ_CK(cudaStreamSynchronize(b->st));
  b->h_sys[slot] = S;
  R.params = h.params;
  R.need_prime = h.pending_prime != 0;
  return PRISMQ_OK;
}

// ---------------------------------------------------------------------------
// Trajectory frames
// ---------------------------------------------------------------------------
prismq_status prismq_batch_frames_configure(prismq_batch* b, int32_t slot, int32_t interval, int32_t capacity,
                                            int32_t with_velocities) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (b->A.fp64) return fail(PRISMQ_E_INVALID, "trajectory frames cover FP32 systems");
  if (interval < 0 || (interval > 0 && capacity < 1)) return fail(PRISMQ_E_INVALID, "interval >= 0, capacity >= 1");
  SlotRec& R = b->slots[slot];
  float4* mem = nullptr;
  if (interval > 0) {
    const size_t bytes = (size_t)capacity * (with_velocities ? 2 : 1) * sizeof(float4) * (size_t)R.n_atoms;
    if (cudaMalloc(&mem, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(PRISMQ_E_CAPACITY, "no device memory for " + std::to_string(capacity) + " frames");
    }
  }
  PQ_CK(cudaStreamSynchronize(b->st));  // no copy into the old ring is still in flight
  if (R.fr_mem) cudaFree(R.fr_mem);
  R.fr_mem = mem;
  R.fr_interval = interval;
  R.fr_cap = interval > 0 ? capacity : 0;
  R.fr_vel = with_velocities ? 1 : 0;
  R.fr_written = R.fr_read = 0;
  R.fr_steps.assign(R.fr_cap, -1);
  return PRISMQ_OK;
}

prismq_status prismq_batch_frames_read(prismq_batch* b, int32_t slot, float* xyz, float* vxyz, int64_t* steps,
                                       int32_t max_frames, int32_t* n_out, int64_t* dropped) {
  prismq_status rc = check_slot(b, slot);
  if (rc != PRISMQ_OK) return rc;
  if (!n_out || max_frames < 0 || (max_frames > 0 && !xyz)) return fail(PRISMQ_E_INVALID, "invalid argument");
  *n_out = 0;
  if (dropped) *dropped = 0;
  SlotRec& R = b->slots[slot];
  if (R.fr_interval <= 0) return fail(PRISMQ_E_INVALID, "no trajectory frames configured");
  if (vxyz && !R.fr_vel) return fail(PRISMQ_E_INVALID, "frames were configured without velocities");
  if (R.fr_written - R.fr_read > R.fr_cap) {  // overwritten before they were read
    if (dropped) *dropped = R.fr_written - R.fr_cap - R.fr_read;
    R.fr_read = R.fr_written - R.fr_cap;
  }
  const int count = (int)std::min<int64_t>(R.fr_written - R.fr_read, max_frames);
  const int n = (int)R.n_atoms;
  for (int i = 0; i < count; ++i) {
    const int64_t sl = (R.fr_read + i) % R.fr_cap;
    const float4* src = R.fr_mem + sl * (R.fr_vel ? 2 : 1) * n;
    k_xyz_to_aos<<<(n + 255) / 256, 256, 0, b->st>>>(b->d_stage, src, n);
    PQ_CK(cudaMemcpyAsync(xyz + (size_t)i * 3 * n, b->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->st));
    if (vxyz) {
      k_xyz_to_aos<<<(n + 255) / 256, 256, 0, b->st>>>(b->d_stage, src + n, n);
      PQ_CK(cudaMemcpyAsync(vxyz + (size_t)i * 3 * n, b->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost,
                            b->st));
    }
    if (steps) steps[i] = R.fr_steps[sl];
  }
  PQ_CK(cudaGetLastError());
  PQ_CK(cudaStreamSynchronize(b->st));
  R.fr_read += count;
  *n_out = count;
  return PRISMQ_OK;
}

prismq_status prismq_frames_configure(prismq_system* sys, int32_t interval, int32_t capacity, int32_t with_velocities) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_frames_configure(sys->b, sys->slot, interval, capacity, with_velocities);
}
prismq_status prismq_frames_read(prismq_system* sys, float* xyz, float* vxyz, int64_t* steps, int32_t max_frames,
                                 int32_t* n_out, int64_t* dropped) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_frames_read(sys->b, sys->slot, xyz, vxyz, steps, max_frames, n_out, dropped);
}

prismq_status prismq_checkpoint_size_for_atoms(int64_t n_atoms, size_t* bytes) {
  if (!bytes || n_atoms < 0) return fail(PRISMQ_E_INVALID, "n_atoms < 0 or bytes NULL");
  *bytes = ckpt_bytes(n_atoms);
  return PRISMQ_OK;
}

prismq_status prismq_checkpoint_size(prismq_system* sys, size_t* bytes) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_checkpoint_size(sys->b, sys->slot, bytes);
}
prismq_status prismq_checkpoint_save(prismq_system* sys, void* buf, size_t cap, size_t* written) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_checkpoint_save(sys->b, sys->slot, buf, cap, written);
}
prismq_status prismq_checkpoint_restore(prismq_system* sys, const void* buf, size_t len) {
  if (!sys) return fail(PRISMQ_E_INVALID, "system is NULL");
  return prismq_batch_checkpoint_restore(sys->b, sys->slot, buf, len);
}

}  // extern "C"

// ===========================================================================
// Hooks for the job server (server.cpp): a job is lowered on the submitting
// thread and admitted, already lowered, by the server's worker thread.
// ===========================================================================
namespace pq {

struct PreparedSystem {
  Lowered L;
  prismq_params p;
};

prismq_status prepare_system(const prismq_topology* t, const prismq_params* p, PreparedSystem** out) {
  if (!out) return fail(PRISMQ_E_INVALID, "NULL argument");
  *out = nullptr;
  prismq_status rc = check_params(p);
  if (rc != PRISMQ_OK) return rc;
  auto* S = new PreparedSystem();
  rc = lower_topology(t, &S->L);
  if (rc != PRISMQ_OK) {
    delete S;
    return rc;
  }
  init_velocities(&S->L, *p);
  S->p = *p;
  *out = S;
  return PRISMQ_OK;
}

void free_prepared(PreparedSystem* s) { delete s; }

int32_t prepared_atoms(const PreparedSystem* s) { return s ? s->L.n : 0; }

prismq_status admit_prepared(prismq_batch* b, const PreparedSystem* s, int32_t* slot) {
  if (!b || !s || !slot) return fail(PRISMQ_E_INVALID, "NULL argument");
  int sl = -1;
  prismq_status rc = batch_admit(b, s->L, s->p, &sl);
  if (rc != PRISMQ_OK) return rc;
  *slot = sl;
  return PRISMQ_OK;
}

// The largest batch (in atoms, a multiple of 32) whose arena fits in
// max_bytes of device memory.
prismq_status batch_create_for_bytes(int64_t max_bytes, int32_t max_systems, prismq_batch** out,
                                     int64_t* atom_cap, int64_t* device_bytes) {
  if (!out || max_bytes <= 0 || max_systems <= 0) return fail(PRISMQ_E_INVALID, "invalid server size");
  int64_t b0 = 0, b1 = 0;
  {
    prismq_batch probe;
    batch_alloc_sized(&probe, 32, max_systems, true, &b0);
    batch_alloc_sized(&probe, 32 + 32 * 1024, max_systems, true, &b1);
  }
  const int64_t per32 = std::max<int64_t>((b1 - b0) / 1024, 1);  // bytes per 32 atoms
  int64_t n = max_bytes > b0 ? 32 + (max_bytes - b0) / per32 * 32 : 0;
  for (; n >= 32; n -= 32) {
    prismq_batch probe;
    int64_t bytes = 0;
    batch_alloc_sized(&probe, n, max_systems, true, &bytes);
    if (bytes <= max_bytes) break;
  }
  if (n < 32)
    return fail(PRISMQ_E_CAPACITY, "max_hbm_bytes holds no arena for " + std::to_string(max_systems) + " systems");
  auto* B = new prismq_batch();
  int64_t bytes = 0;
  prismq_status rc = batch_alloc_sized(B, n, max_systems, false, &bytes);
  if (rc != PRISMQ_OK) {
    delete B;
    return rc;
  }
  *out = B;
  if (atom_cap) *atom_cap = n;
  if (device_bytes) *device_bytes = bytes;
  return PRISMQ_OK;
}

}  // namespace pq
