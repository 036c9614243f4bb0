/*
 * CPU oracle for the Prism-Q classical MD step — TEST INFRASTRUCTURE ONLY
 * (tests, __graft_entry__.smoke()'s checker, bench.py's CPU baseline leg).
 * The product library never links or calls this file.
 *
 * A plain-C restatement of the reference algorithm.  Every function cites the
 * reference lines it follows (paths relative to the Delfictus/Prism-Q tree).
 * Compiled with -ffp-contract=off so float expressions are evaluated exactly
 * as written; FP32 sections therefore reproduce the library's integrator bit
 * for bit, and the FP64 force oracle measures the library's arithmetic error.
 */
#include "prismq_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_COULOMB 332.0636f                 /* nhs_amber_fused.cu:64 */
#define ORC_AKMA 418.4f                       /* :67 AMBER_KCAL_TO_AMU_A2_PS2 */
#define ORC_KB 0.001987204f                   /* :68 */
#define ORC_MAXF 1000.0f                      /* :69 MAX_INTEGRATOR_FORCE_KCAL_MOL_A */
#define ORC_CELL 10.0f                        /* :167 CELL_SIZE */
#define ORC_CELL_INV 0.1f                     /* :168 CELL_SIZE_INV */
#define ORC_ROW_CAP 1024                      /* :172 NEIGHBOR_LIST_SIZE */
#define ORC_FIX_INV 2.3283064365386963e-10f   /* 2^-32 */
#define ORC_FIX_SCALE 4294967296.0f           /* 2^32 */

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, Salmon et al. SC'11; key (seed, stream), counter (atom,
 * step_lo, step_hi16|purpose8|epoch8, 0): scripts/physics_refs/rng_streams.py:62-84 */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The injected-noise definition: Box–Muller over Philox words with
 * ln(u) = e·ln2 + 2·atanh((m-1)/(m+1)) and sin/cos by Taylor series on
 * [0, π/4] — only exact IEEE operations and fmaf, so identical everywhere. */
static float fbits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t bitsf(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static float orc_log_unit(float u) {
  const uint32_t b = bitsf(u);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = fbits((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = fmaf(s2, 0.11111111f, 0.14285715f);
  p = fmaf(s2, p, 0.2f);
  p = fmaf(s2, p, 0.33333334f);
  p = fmaf(s2, p, 1.0f);
  const float two_s = s + s;
  return fmaf((float)e, 0.69314718f, two_s * p);
}

static void orc_sincos_oct(float t, float* sn, float* cs) {
  const float t2 = t * t;
  float ps = fmaf(t2, 2.7557319e-06f, -1.9841270e-04f);
  ps = fmaf(t2, ps, 8.3333333e-03f);
  ps = fmaf(t2, ps, -1.6666667e-01f);
  ps = fmaf(t2, ps, 1.0f);
  float pc = fmaf(t2, -2.7557319e-07f, 2.4801587e-05f);
  pc = fmaf(t2, pc, -1.3888889e-03f);
  pc = fmaf(t2, pc, 4.1666667e-02f);
  pc = fmaf(t2, pc, -0.5f);
  pc = fmaf(t2, pc, 1.0f);
  *sn = t * ps;
  *cs = pc;
}

static void orc_turn(float u, float* c, float* s) {
  const float t = u * 4.0f;
  const int q = (int)t;
  float f = t - (float)q;
  const int flip = f > 0.5f;
  if (flip) f = 1.0f - f;
  float sn, cs;
  orc_sincos_oct(f * 1.57079633f, &sn, &cs);
  if (flip) { const float tmp = sn; sn = cs; cs = tmp; }
  switch (q & 3) {
    case 0: *c = cs; *s = sn; break;
    case 1: *c = -sn; *s = cs; break;
    case 2: *c = -cs; *s = -sn; break;
    default: *c = sn; *s = -cs; break;
  }
}

void orc_normal3(uint32_t seed, uint32_t stream, uint32_t atom, uint64_t step, uint32_t purpose,
                 float out[3]) {
  const uint32_t ctr[4] = {atom, (uint32_t)(step & 0xffffffffu),
                           ((uint32_t)((step >> 32) & 0xffffu) << 16) | ((purpose & 0xffu) << 8), 0u};
  const uint32_t key[2] = {seed, stream};
  uint32_t r[4];
  orc_philox4x32_10(ctr, key, r);
  const float inv24 = 5.9604645e-08f;
  const float u1 = (float)((r[0] >> 8) + 1u) * inv24;
  const float u2 = (float)(r[1] >> 8) * inv24;
  const float u3 = (float)((r[2] >> 8) + 1u) * inv24;
  const float u4 = (float)(r[3] >> 8) * inv24;
  const float ra = sqrtf(-2.0f * orc_log_unit(u1));
  const float rb = sqrtf(-2.0f * orc_log_unit(u3));
  float ca, sa, cb, sb;
  orc_turn(u2, &ca, &sa);
  orc_turn(u4, &cb, &sb);
  out[0] = ra * ca;
  out[1] = ra * sa;
  out[2] = rb * cb;
  (void)sb;
}

static int64_t orc_f2fixed(float v) {
  const float s = v * ORC_FIX_SCALE;
  if (s != s) return 0;
  if (s >= 9.2233720368547758e18f) return INT64_MAX;
  if (s <= -9.2233720368547758e18f) return INT64_MIN;
  return (int64_t)llrintf(s);
}
static float orc_fixed2f(int64_t v) { return (float)v * ORC_FIX_INV; }

/* ------------------------------------------------------------------------ */
/* Neighbour schemes.
 * Reference grid: fused_engine.rs:12285-12330 (origin = bbox_min - 10,
 * n = ceil((extent + 20)/10)); cell index: nhs_amber_fused.cu:11704-11717
 * ((int)((x - o) * 0.1f) then clamp); 27-cell stencil and the `!(r2 > cutoff_sq)`
 * keep rule: nhs_neighbor_warp.cuh:42-76.  r2 is evaluated as
 * (dx*dx + dy*dy) + dz*dz, the order of scripts/physics_refs/neighbor_list.py:63-91. */
static float r2_plain(float dx, float dy, float dz) {
  const float a = dx * dx;
  const float b = dy * dy;
  const float c = dz * dz;
  return (a + b) + c;
}

static int excluded(int i, int j, const int32_t* off, const int32_t* lst) {
  if (!off) return 0;
  for (int q = off[i]; q < off[i + 1]; ++q)
    if (lst[q] == j) return 1;
  return 0;
}

typedef struct {
  float origin[3];
  int dims[3];
} orc_grid;

static orc_grid grid_from(int n, const float* pos) {
  orc_grid g;
  for (int d = 0; d < 3; ++d) {
    float lo = pos[d], hi = pos[d];
    for (int a = 1; a < n; ++a) {
      const float v = pos[3 * a + d];
      if (v < lo) lo = v;
      if (v > hi) hi = v;
    }
    g.origin[d] = lo - ORC_CELL;
    const float extent = (hi - lo) + 2.0f * ORC_CELL;
    long v = (long)ceilf(extent / ORC_CELL);
    g.dims[d] = (int)(v < 1 ? 1 : v);
  }
  return g;
}

static int cell_of(const orc_grid* g, const float* p) {
  int ix[3];
  for (int d = 0; d < 3; ++d) {
    int c = (int)((p[d] - g->origin[d]) * ORC_CELL_INV);
    if (c < 0) c = 0;
    if (c > g->dims[d] - 1) c = g->dims[d] - 1;
    ix[d] = c;
  }
  return ix[0] + ix[1] * g->dims[0] + ix[2] * g->dims[0] * g->dims[1];
}

/* counting sort of atoms into cells; returns start[ncell+1] and members[n] (ascending) */
static void cell_sort(int n, const float* pos, const orc_grid* g, int** start_out, int** mem_out,
                      int* occ) {
  const long ncell = (long)g->dims[0] * g->dims[1] * g->dims[2];
  int* start = (int*)calloc((size_t)ncell + 1, sizeof(int));
  int* mem = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int* cell = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int a = 0; a < n; ++a) {
    cell[a] = cell_of(g, pos + 3 * a);
    start[cell[a] + 1]++;
  }
  int mx = 0;
  for (long c = 0; c < ncell; ++c) {
    if (start[c + 1] > mx) mx = start[c + 1];
    start[c + 1] += start[c];
  }
  int* cur = (int*)malloc(sizeof(int) * (size_t)ncell);
  for (long c = 0; c < ncell; ++c) cur[c] = start[c];
  for (int a = 0; a < n; ++a) mem[cur[cell[a]]++] = a;
  free(cur);
  free(cell);
  if (occ) *occ = mx;
  *start_out = start;
  *mem_out = mem;
}

/* REF27 rows of atom i (unsorted), rule !(r2 > r2max); returns row length or -1 on overflow */
static int ref27_row(int i, const float* pos, const orc_grid* g, const int* start, const int* mem,
                     float r2max, const int32_t* eo, const int32_t* el, int* row, int cap) {
  const int c = cell_of(g, pos + 3 * i);
  const int cx = c % g->dims[0], cy = (c / g->dims[0]) % g->dims[1], cz = c / (g->dims[0] * g->dims[1]);
  int cnt = 0;
  for (int dz = -1; dz <= 1; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= g->dims[2]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= g->dims[1]) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        const int x = cx + dx;
        if (x < 0 || x >= g->dims[0]) continue;
        const int cc = x + y * g->dims[0] + z * g->dims[0] * g->dims[1];
        for (int k = start[cc]; k < start[cc + 1]; ++k) {
          const int j = mem[k];
          if (j == i) continue;
          const float r2 = r2_plain(pos[3 * j] - pos[3 * i], pos[3 * j + 1] - pos[3 * i + 1],
                                    pos[3 * j + 2] - pos[3 * i + 2]);
          if (r2 > r2max) continue;
          if (excluded(i, j, eo, el)) continue;
          if (cnt >= cap) return -1;
          row[cnt++] = j;
        }
      }
    }
  }
  return cnt;
}

static int cmp_int(const void* a, const void* b) {
  const int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

long orc_pairs_ref27(int n, const float* pos, const float* grid_pos, float r2max, const int32_t* excl_off,
                     const int32_t* excl, int32_t* out, long cap, int* max_occupancy) {
  const orc_grid g = grid_from(n, grid_pos);
  int *start, *mem;
  cell_sort(n, pos, &g, &start, &mem, max_occupancy);
  int* row = (int*)malloc(sizeof(int) * 8192);
  long total = 0;
  for (int i = 0; i < n; ++i) {
    const int cnt = ref27_row(i, pos, &g, start, mem, r2max, excl_off, excl, row, 8192);
    if (cnt < 0) { total = -1; break; }
    qsort(row, (size_t)cnt, sizeof(int), cmp_int);
    for (int k = 0; k < cnt; ++k) {
      if (row[k] <= i) continue;
      if (total < cap && out) {
        out[2 * total] = i;
        out[2 * total + 1] = row[k];
      }
      ++total;
    }
  }
  free(row);
  free(start);
  free(mem);
  return total;
}

long orc_pairs_brute(int n, const float* pos, float r2max, const int32_t* excl_off, const int32_t* excl,
                     int32_t* out, long cap) {
  /* rows counted in parallel, then written at their prefix offsets: the
   * output is the sequential (i, then j) order */
  long* cnt = (long*)calloc((size_t)n + 1, sizeof(long));
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) {
    long c = 0;
    for (int j = i + 1; j < n; ++j) {
      const float r2 = r2_plain(pos[3 * j] - pos[3 * i], pos[3 * j + 1] - pos[3 * i + 1],
                                pos[3 * j + 2] - pos[3 * i + 2]);
      if (r2 > r2max) continue;
      if (excluded(i, j, excl_off, excl)) continue;
      ++c;
    }
    cnt[i + 1] = c;
  }
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  const long total = cnt[n];
  if (out) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
      long k = cnt[i];
      if (k >= cap) continue;
      for (int j = i + 1; j < n && k < cap; ++j) {
        const float r2 = r2_plain(pos[3 * j] - pos[3 * i], pos[3 * j + 1] - pos[3 * i + 1],
                                  pos[3 * j + 2] - pos[3 * i + 2]);
        if (r2 > r2max) continue;
        if (excluded(i, j, excl_off, excl)) continue;
        out[2 * k] = i;
        out[2 * k + 1] = j;
        ++k;
      }
    }
  }
  free(cnt);
  return total;
}

/* ------------------------------------------------------------------------ */
/* System lowering, following NhsAmberFusedEngine::new_on_stream_with_nonbonded_policy:
 * pairs14 CSR from exact exceptions, both directions, ascending partner, last
 * definition wins (fused_engine.rs:11625-11680); exclusion CSR = topology
 * exclusions minus pairs14 partners (:11680-11700); incidence sorted by
 * (term, position) (:11704-11745, :16034-16063). */
typedef struct {
  int central, h[3], nh;
  float len[3], imc, imh;
} orc_cluster;

struct orc_sys {
  int n;
  orc_params p;
  float *x, *v, *m, *q, *sig, *eps;
  float* x0; /* construction positions (fixed reference grid) */
  int *p14_off, *p14_j;
  float *p14_qq, *p14_sig, *p14_eps;
  int *ex_off, *ex_list;  /* ordinary exclusions (minus pairs14) */
  int *all_off, *all_list; /* exclusions ∪ pairs14 (pairs never evaluated as ordinary) */
  int nb, na, nd;
  prismq_bond* bonds;
  prismq_angle* angles;
  prismq_dihedral* dihs;
  int *ib_off, *ib, *ia_off, *ia, *id_off, *id;
  int ncl;
  orc_cluster* cl;
  int* in_cluster;
  long long step;
  /* REF27 rows cache */
  int* rows;
  int* rowlen;
  /* run protocol: parameters of each step from the director restatement */
  int proto_on;
  prismq_protocol proto;
  long long proto_origin; /* director step = step - proto_origin */
};

int orc_n_atoms(const orc_sys* s) { return s->n; }
long long orc_step_count(const orc_sys* s) { return s->step; }

static int* build_csr(int n, int** lists, int* lens, int** flat) {
  int* off = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  off[0] = 0;
  for (int a = 0; a < n; ++a) off[a + 1] = off[a] + lens[a];
  *flat = (int*)malloc(sizeof(int) * (size_t)(off[n] > 0 ? off[n] : 1));
  for (int a = 0; a < n; ++a)
    if (lens[a]) memcpy(*flat + off[a], lists[a], sizeof(int) * (size_t)lens[a]);
  return off;
}

typedef struct {
  int j;
  float qq, sig, eps;
} p14e;
static int cmp_p14(const void* a, const void* b) {
  const p14e *x = (const p14e*)a, *y = (const p14e*)b;
  return (x->j > y->j) - (x->j < y->j);
}

orc_sys* orc_create(const prismq_topology* t, const orc_params* p) {
  const int n = t->n_atoms;
  orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
  s->n = n;
  s->p = *p;
  s->x = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  s->v = (float*)calloc(3 * (size_t)n, sizeof(float));
  s->x0 = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  memcpy(s->x, t->positions, sizeof(float) * 3 * (size_t)n);
  memcpy(s->x0, t->positions, sizeof(float) * 3 * (size_t)n);
  s->m = (float*)malloc(sizeof(float) * (size_t)n);
  s->q = (float*)malloc(sizeof(float) * (size_t)n);
  s->sig = (float*)malloc(sizeof(float) * (size_t)n);
  s->eps = (float*)malloc(sizeof(float) * (size_t)n);
  memcpy(s->m, t->masses, sizeof(float) * (size_t)n);
  memcpy(s->q, t->charges, sizeof(float) * (size_t)n);
  memcpy(s->sig, t->lj_sigma, sizeof(float) * (size_t)n);
  memcpy(s->eps, t->lj_epsilon, sizeof(float) * (size_t)n);
  /* pairs14 */
  int* cnt = (int*)calloc((size_t)n, sizeof(int));
  for (int e = 0; e < t->n_exceptions; ++e) {
    cnt[t->exceptions[e].i]++;
    cnt[t->exceptions[e].j]++;
  }
  p14e** rows = (p14e**)malloc(sizeof(p14e*) * (size_t)n);
  int* fill = (int*)calloc((size_t)n, sizeof(int));
  for (int a = 0; a < n; ++a) rows[a] = (p14e*)malloc(sizeof(p14e) * (size_t)(cnt[a] + 1));
  for (int e = 0; e < t->n_exceptions; ++e) {
    const prismq_exception* x = &t->exceptions[e];
    const int ends[2][2] = {{x->i, x->j}, {x->j, x->i}};
    for (int k = 0; k < 2; ++k) {
      const int a = ends[k][0], b = ends[k][1];
      int found = -1;
      for (int q = 0; q < fill[a]; ++q)
        if (rows[a][q].j == b) found = q;
      p14e v = {b, x->charge_product, x->sigma, x->epsilon};
      if (found >= 0) rows[a][found] = v; else rows[a][fill[a]++] = v;
    }
  }
  s->p14_off = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  s->p14_off[0] = 0;
  for (int a = 0; a < n; ++a) {
    qsort(rows[a], (size_t)fill[a], sizeof(p14e), cmp_p14);
    s->p14_off[a + 1] = s->p14_off[a] + fill[a];
  }
  const int np14 = s->p14_off[n];
  s->p14_j = (int*)malloc(sizeof(int) * (size_t)(np14 + 1));
  s->p14_qq = (float*)malloc(sizeof(float) * (size_t)(np14 + 1));
  s->p14_sig = (float*)malloc(sizeof(float) * (size_t)(np14 + 1));
  s->p14_eps = (float*)malloc(sizeof(float) * (size_t)(np14 + 1));
  for (int a = 0; a < n; ++a)
    for (int q = 0; q < fill[a]; ++q) {
      const int k = s->p14_off[a] + q;
      s->p14_j[k] = rows[a][q].j;
      s->p14_qq[k] = rows[a][q].qq;
      s->p14_sig[k] = rows[a][q].sig;
      s->p14_eps[k] = rows[a][q].eps;
    }
  /* exclusions minus pairs14; and exclusions ∪ pairs14 */
  int** el = (int**)malloc(sizeof(int*) * (size_t)n);
  int** al = (int**)malloc(sizeof(int*) * (size_t)n);
  int* elen = (int*)calloc((size_t)n, sizeof(int));
  int* alen = (int*)calloc((size_t)n, sizeof(int));
  for (int a = 0; a < n; ++a) {
    const int b0 = t->exclusion_offsets ? t->exclusion_offsets[a] : 0;
    const int b1 = t->exclusion_offsets ? t->exclusion_offsets[a + 1] : 0;
    el[a] = (int*)malloc(sizeof(int) * (size_t)(b1 - b0 + 1));
    al[a] = (int*)malloc(sizeof(int) * (size_t)(b1 - b0 + fill[a] + 1));
    for (int q = b0; q < b1; ++q) {
      const int j = t->exclusions[q];
      int is14 = 0;
      for (int r = 0; r < fill[a]; ++r)
        if (rows[a][r].j == j) is14 = 1;
      if (!is14) el[a][elen[a]++] = j;
      al[a][alen[a]++] = j;
    }
    for (int r = 0; r < fill[a]; ++r) {
      int dup = 0;
      for (int q = 0; q < alen[a]; ++q)
        if (al[a][q] == rows[a][r].j) dup = 1;
      if (!dup) al[a][alen[a]++] = rows[a][r].j;
    }
  }
  s->ex_off = build_csr(n, el, elen, &s->ex_list);
  s->all_off = build_csr(n, al, alen, &s->all_list);
  for (int a = 0; a < n; ++a) {
    free(el[a]);
    free(al[a]);
    free(rows[a]);
  }
  free(el); free(al); free(elen); free(alen); free(rows); free(fill); free(cnt);
  /* bonded terms and incidence (term index order; position order within a term) */
  s->nb = t->n_bonds;
  s->na = t->n_angles;
  s->nd = t->n_dihedrals;
  s->bonds = (prismq_bond*)malloc(sizeof(prismq_bond) * (size_t)(s->nb + 1));
  s->angles = (prismq_angle*)malloc(sizeof(prismq_angle) * (size_t)(s->na + 1));
  s->dihs = (prismq_dihedral*)malloc(sizeof(prismq_dihedral) * (size_t)(s->nd + 1));
  if (s->nb) memcpy(s->bonds, t->bonds, sizeof(prismq_bond) * (size_t)s->nb);
  if (s->na) memcpy(s->angles, t->angles, sizeof(prismq_angle) * (size_t)s->na);
  if (s->nd) memcpy(s->dihs, t->dihedrals, sizeof(prismq_dihedral) * (size_t)s->nd);
  {
    /* (atom, term*4+position) entries in term order give rows sorted by (term, position) */
    const int nterm[3] = {s->nb, s->na, s->nd};
    int** offs[3] = {&s->ib_off, &s->ia_off, &s->id_off};
    int** lists[3] = {&s->ib, &s->ia, &s->id};
    for (int kind = 0; kind < 3; ++kind) {
      int* off = (int*)calloc((size_t)n + 1, sizeof(int));
      for (int pass = 0; pass < 2; ++pass) {
        int* cur = NULL;
        if (pass == 1) {
          for (int a = 0; a < n; ++a) off[a + 1] += off[a];
          *lists[kind] = (int*)malloc(sizeof(int) * (size_t)(off[n] + 1));
          cur = (int*)malloc(sizeof(int) * (size_t)(n + 1));
          memcpy(cur, off, sizeof(int) * (size_t)n);
        }
        for (int k = 0; k < nterm[kind]; ++k) {
          int at[4], na = 0;
          if (kind == 0) { at[0] = s->bonds[k].i; at[1] = s->bonds[k].j; na = 2; }
          if (kind == 1) { at[0] = s->angles[k].i; at[1] = s->angles[k].j; at[2] = s->angles[k].k; na = 3; }
          if (kind == 2) {
            at[0] = s->dihs[k].i; at[1] = s->dihs[k].j; at[2] = s->dihs[k].k; at[3] = s->dihs[k].l; na = 4;
          }
          for (int p = 0; p < na; ++p) {
            if (pass == 0) off[at[p] + 1]++;
            else (*lists[kind])[cur[at[p]]++] = k * 4 + p;
          }
        }
        free(cur);
      }
      *offs[kind] = off;
    }
  }
  /* clusters */
  s->ncl = t->n_clusters;
  s->cl = (orc_cluster*)malloc(sizeof(orc_cluster) * (size_t)(s->ncl + 1));
  s->in_cluster = (int*)calloc((size_t)n, sizeof(int));
  for (int c = 0; c < s->ncl; ++c) {
    const prismq_hcluster* h = &t->clusters[c];
    orc_cluster* o = &s->cl[c];
    o->central = h->central_atom;
    o->nh = h->n_hydrogens;
    o->imc = h->inv_mass_central;
    o->imh = h->inv_mass_h;
    for (int k = 0; k < 3; ++k) {
      o->h[k] = h->hydrogen_atoms[k];
      o->len[k] = h->bond_lengths[k];
    }
  }
  s->rows = (int*)malloc(sizeof(int) * (size_t)n * ORC_ROW_CAP);
  s->rowlen = (int*)calloc((size_t)n, sizeof(int));
  return s;
}

void orc_destroy(orc_sys* s) {
  if (!s) return;
  void* ptrs[] = {s->x, s->v, s->m, s->q, s->sig, s->eps, s->x0, s->p14_off, s->p14_j, s->p14_qq,
                  s->p14_sig, s->p14_eps, s->ex_off, s->ex_list, s->all_off, s->all_list, s->bonds,
                  s->angles, s->dihs, s->ib_off, s->ib, s->ia_off, s->ia, s->id_off, s->id, s->cl,
                  s->in_cluster, s->rows, s->rowlen};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
  free(s);
}

void orc_set_state(orc_sys* s, const float* x, const float* v) {
  if (x) memcpy(s->x, x, sizeof(float) * 3 * (size_t)s->n);
  if (v) memcpy(s->v, v, sizeof(float) * 3 * (size_t)s->n);
}
void orc_get_state(const orc_sys* s, float* x, float* v) {
  if (x) memcpy(x, s->x, sizeof(float) * 3 * (size_t)s->n);
  if (v) memcpy(v, s->v, sizeof(float) * 3 * (size_t)s->n);
}

int orc_ref_exclusions(const orc_sys* s, int32_t* off, int32_t* list, long cap) {
  const int tot = s->ex_off[s->n];
  if (cap < tot) return -tot;
  memcpy(off, s->ex_off, sizeof(int) * (size_t)(s->n + 1));
  if (tot) memcpy(list, s->ex_list, sizeof(int) * (size_t)tot);
  return tot;
}

/* ------------------------------------------------------------------------ */
/* Force laws, FP32 — compute_bond_force :355, compute_angle_force :389,
 * compute_dihedral_force :525, compute_nonbonded_force :644. */
static void bond_f32(const float* x, const prismq_bond* b, float fi[3], float fj[3], double* e) {
  const float rx = x[3 * b->j] - x[3 * b->i], ry = x[3 * b->j + 1] - x[3 * b->i + 1],
              rz = x[3 * b->j + 2] - x[3 * b->i + 2];
  const float r = sqrtf(rx * rx + ry * ry + rz * rz);
  if (r < 1e-8f) return;
  const float dr = r - b->r0;
  const float fm = -2.0f * b->k * dr / r;
  const float f[3] = {fm * rx, fm * ry, fm * rz};
  for (int d = 0; d < 3; ++d) { fi[d] -= f[d]; fj[d] += f[d]; }
  if (e) *e += (double)b->k * (double)dr * (double)dr * 0.5;
}

static void angle_f32(const float* x, const prismq_angle* a, float fi[3], float fj[3], float fk[3],
                      double* e) {
  const float* pi = x + 3 * a->i;
  const float* pj = x + 3 * a->j;
  const float* pk = x + 3 * a->k;
  const float rij[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
  const float rkj[3] = {pk[0] - pj[0], pk[1] - pj[1], pk[2] - pj[2]};
  const float li = sqrtf(rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
  const float lk = sqrtf(rkj[0] * rkj[0] + rkj[1] * rkj[1] + rkj[2] * rkj[2]);
  if (li < 1e-8f || lk < 1e-8f) return;
  float c = (rij[0] * rkj[0] + rij[1] * rkj[1] + rij[2] * rkj[2]) / (li * lk);
  c = fmaxf(-1.0f, fminf(1.0f, c));
  const float th = acosf(c);
  const float dth = th - a->theta0;
  float sn = sqrtf(1.0f - c * c);
  if (sn < 1e-8f) sn = 1e-8f;
  const float fm = -2.0f * a->force_k * dth / sn;
  const float ii = 1.0f / li, ik = 1.0f / lk;
  for (int d = 0; d < 3; ++d) {
    const float di = (rkj[d] * ik - c * rij[d] * ii) * ii;
    const float dk = (rij[d] * ii - c * rkj[d] * ik) * ik;
    fi[d] -= fm * di;
    fk[d] -= fm * dk;
    fj[d] += fm * (di + dk);
  }
  if (e) *e += (double)a->force_k * (double)dth * (double)dth * (1.0 / 3.0);
}

static void dihedral_f32(const float* x, const prismq_dihedral* t, float f0[3], float f1[3], float f2[3],
                         float f3[3], double* e) {
  const float* pi = x + 3 * t->i;
  const float* pj = x + 3 * t->j;
  const float* pk = x + 3 * t->k;
  const float* pl = x + 3 * t->l;
  const float v0[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
  const float v1[3] = {pk[0] - pj[0], pk[1] - pj[1], pk[2] - pj[2]};
  const float v2[3] = {pk[0] - pl[0], pk[1] - pl[1], pk[2] - pl[2]};
  const float c0[3] = {v0[1] * v1[2] - v0[2] * v1[1], v0[2] * v1[0] - v0[0] * v1[2], v0[0] * v1[1] - v0[1] * v1[0]};
  const float c1[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  const float n1 = c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2];
  const float n2 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
  const float nb = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
  if (n1 < 1e-16f || n2 < 1e-16f || nb < 1e-16f) return;
  const float lbc = sqrtf(nb);
  float cp = (c0[0] * c1[0] + c0[1] * c1[1] + c0[2] * c1[2]) / sqrtf(n1 * n2);
  cp = fmaxf(-1.0f, fminf(1.0f, cp));
  float phi;
  if (cp > 0.99f || cp < -0.99f) {
    const float xc[3] = {c0[1] * c1[2] - c0[2] * c1[1], c0[2] * c1[0] - c0[0] * c1[2], c0[0] * c1[1] - c0[1] * c1[0]};
    float s2 = (xc[0] * xc[0] + xc[1] * xc[1] + xc[2] * xc[2]) / (n1 * n2);
    s2 = fmaxf(0.0f, fminf(1.0f, s2));
    phi = asinf(sqrtf(s2));
    if (cp < 0.0f) phi = 3.14159265358979323846f - phi;
  } else {
    phi = acosf(cp);
  }
  if (v0[0] * c1[0] + v0[1] * c1[1] + v0[2] * c1[2] < 0.0f) phi = -phi;
  const float nn = (float)t->periodicity;
  const float dE = -t->force_k * nn * sinf(nn * phi - t->phase);
  const float inb = 1.0f / nb;
  const float ff0 = (-dE * lbc) / n1;
  const float ff1 = (v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2]) * inb;
  const float ff2 = (v2[0] * v1[0] + v2[1] * v1[1] + v2[2] * v1[2]) * inb;
  const float ff3 = (dE * lbc) / n2;
  for (int d = 0; d < 3; ++d) {
    const float a1 = ff0 * c0[d], a4 = ff3 * c1[d];
    const float sv = ff1 * a1 - ff2 * a4;
    f0[d] += a1;
    f1[d] += sv - a1;
    f2[d] += -sv - a4;
    f3[d] += a4;
  }
  if (e) *e += (double)t->force_k * (1.0 + cos((double)nn * (double)phi - (double)t->phase)) * 0.25;
}

/* r2 of the force phase: fmaf(dz,dz,fmaf(dy,dy,dx*dx)) with d = xj - xi.  This is
 * the rule that decides which pairs lie inside the cutoff, for both oracles. */
static float r2_force(const float* x, int i, int j, float* d) {
  d[0] = x[3 * j] - x[3 * i];
  d[1] = x[3 * j + 1] - x[3 * i + 1];
  d[2] = x[3 * j + 2] - x[3 * i + 2];
  return fmaf(d[2], d[2], fmaf(d[1], d[1], d[0] * d[0]));
}

/* Build REF27 rows for every atom at the current positions (ascending rows,
 * reference nhs_neighbor_warp.cuh:85-113), cutoff^2 * 1.44 (fused_engine.rs:16674). */
static int build_rows(orc_sys* s) {
  const orc_grid g = grid_from(s->n, s->x0);
  int *start, *mem, occ = 0;
  cell_sort(s->n, s->x, &g, &start, &mem, &occ);
  const float r2max = (s->p.cutoff * s->p.cutoff) * 1.44f;
  int bad = occ > 512;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s->n; ++i) {
    int* row = s->rows + (size_t)i * ORC_ROW_CAP;
    const int c = ref27_row(i, s->x, &g, start, mem, r2max, s->ex_off, s->ex_list, row, ORC_ROW_CAP);
    if (c < 0) {
      bad = 1;
      s->rowlen[i] = 0;
      continue;
    }
    qsort(row, (size_t)c, sizeof(int), cmp_int);
    s->rowlen[i] = c;
  }
  free(start);
  free(mem);
  return bad ? -1 : 0;
}

/* The reference force phase, FP32 per-atom gather (nhs_amber_fused.cu:2993-3484). */
static void gather_f32(const orc_sys* s, int i, float out[3], double e[5]) {
  float lf[3] = {0, 0, 0};
  const float* x = s->x;
  for (int q = s->ib_off[i]; q < s->ib_off[i + 1]; ++q) {
    const int ent = s->ib[q];
    const prismq_bond* b = &s->bonds[ent >> 2];
    float fi[3] = {0, 0, 0}, fj[3] = {0, 0, 0};
    bond_f32(x, b, fi, fj, e ? &e[0] : NULL);
    const float* mine = (ent & 3) == 0 ? fi : fj;
    for (int d = 0; d < 3; ++d) lf[d] += mine[d];
  }
  for (int q = s->ia_off[i]; q < s->ia_off[i + 1]; ++q) {
    const int ent = s->ia[q];
    float fi[3] = {0, 0, 0}, fj[3] = {0, 0, 0}, fk[3] = {0, 0, 0};
    angle_f32(x, &s->angles[ent >> 2], fi, fj, fk, e ? &e[1] : NULL);
    const int p = ent & 3;
    const float* mine = p == 0 ? fi : (p == 1 ? fj : fk);
    for (int d = 0; d < 3; ++d) lf[d] += mine[d];
  }
  for (int q = s->id_off[i]; q < s->id_off[i + 1]; ++q) {
    const int ent = s->id[q];
    float a[3] = {0, 0, 0}, b[3] = {0, 0, 0}, c[3] = {0, 0, 0}, d4[3] = {0, 0, 0};
    dihedral_f32(x, &s->dihs[ent >> 2], a, b, c, d4, e ? &e[2] : NULL);
    const int p = ent & 3;
    const float* mine = p == 0 ? a : (p == 1 ? b : (p == 2 ? c : d4));
    for (int d = 0; d < 3; ++d) lf[d] += mine[d];
  }
  const float cut2 = s->p.cutoff * s->p.cutoff;
  const float inv_rc = 1.0f / sqrtf(cut2);
  const int* row = s->rows + (size_t)i * ORC_ROW_CAP;
  for (int k = 0; k < s->rowlen[i]; ++k) {
    const int j = row[k];
    int is14 = 0;
    for (int p = s->p14_off[i]; p < s->p14_off[i + 1]; ++p)
      if (s->p14_j[p] == j) { is14 = 1; break; }
    if (is14) continue;
    float d[3];
    const float r2 = r2_force(x, i, j, d);
    if (r2 >= cut2 || r2 < 0.01f) continue;
    const float inv_r = 1.0f / sqrtf(r2);
    const float inv_r2 = inv_r * inv_r;
    const float sigma = 0.5f * (s->sig[i] + s->sig[j]);
    const float eps = sqrtf(s->eps[i] * s->eps[j]);
    const float qq = s->q[i] * s->q[j];
    const float sr = sigma * inv_r, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    const float flj = 24.0f * eps * inv_r2 * (2.0f * sr12 - sr6);
    const float fc = ORC_COULOMB * qq * inv_r2 * inv_r;
    const float tf = flj + fc;
    for (int c = 0; c < 3; ++c) lf[c] -= tf * d[c];
    if (e) {
      const float src = sigma * inv_rc, src2 = src * src, src6 = src2 * src2 * src2, src12 = src6 * src6;
      const double off = 4.0 * (double)eps * ((double)src12 - (double)src6) +
                         (double)ORC_COULOMB * (double)qq * (double)inv_rc;
      const double v = 4.0 * (double)eps * ((double)sr12 - (double)sr6) +
                       (double)ORC_COULOMB * (double)qq * (double)inv_r - off;
      e[4] += v * 0.5;
    }
  }
  for (int p = s->p14_off[i]; p < s->p14_off[i + 1]; ++p) {
    const int j = s->p14_j[p];
    float d[3];
    const float r2 = r2_force(x, i, j, d);
    if (r2 < 1e-8f) continue;
    const float inv_r = 1.0f / sqrtf(r2);
    const float inv_r2 = inv_r * inv_r;
    const float sigma = s->p14_sig[p], eps = s->p14_eps[p], qq = s->p14_qq[p];
    const float sr = sigma * inv_r, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    const float flj = 24.0f * eps * inv_r2 * (2.0f * sr12 - sr6);
    const float fc = ORC_COULOMB * qq * inv_r2 * inv_r;
    const float tf = flj + fc;
    for (int c = 0; c < 3; ++c) lf[c] -= tf * d[c];
    if (e) {
      const double v = 4.0 * (double)eps * ((double)sr12 - (double)sr6) +
                       (double)ORC_COULOMB * (double)qq * (double)inv_r;
      e[3] += v * 0.5;
    }
  }
  out[0] = lf[0];
  out[1] = lf[1];
  out[2] = lf[2];
}

static int forces_f32_impl(orc_sys* s, float* f, double* e5, int rebuild) {
  if (rebuild && build_rows(s) != 0) return 3;
  double tot[5] = {0, 0, 0, 0, 0};
  if (e5) {
    /* serial energy sum in atom order */
    for (int i = 0; i < s->n; ++i) {
      double e[5] = {0, 0, 0, 0, 0};
      gather_f32(s, i, f + 3 * i, e);
      for (int c = 0; c < 5; ++c) tot[c] += e[c];
    }
    for (int c = 0; c < 5; ++c) e5[c] = tot[c];
  } else {
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < s->n; ++i) gather_f32(s, i, f + 3 * i, NULL);
  }
  return 0;
}

int orc_forces_ref_f32(orc_sys* s, float* f, double* e5, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  return forces_f32_impl(s, f, e5, 1);
}

/* ------------------------------------------------------------------------ */
/* FP64 oracle. */
static void bond_f64(const double* x, const prismq_bond* b, double fi[3], double fj[3], double* e) {
  double r[3];
  for (int d = 0; d < 3; ++d) r[d] = x[3 * b->j + d] - x[3 * b->i + d];
  const double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  if (rl < 1e-8) return;
  const double dr = rl - (double)b->r0;
  const double fm = -2.0 * (double)b->k * dr / rl;
  for (int d = 0; d < 3; ++d) { fi[d] -= fm * r[d]; fj[d] += fm * r[d]; }
  *e += (double)b->k * dr * dr;
}

static void angle_f64(const double* x, const prismq_angle* a, double fi[3], double fj[3], double fk[3],
                      double* e) {
  double rij[3], rkj[3];
  for (int d = 0; d < 3; ++d) {
    rij[d] = x[3 * a->i + d] - x[3 * a->j + d];
    rkj[d] = x[3 * a->k + d] - x[3 * a->j + d];
  }
  const double li = sqrt(rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
  const double lk = sqrt(rkj[0] * rkj[0] + rkj[1] * rkj[1] + rkj[2] * rkj[2]);
  if (li < 1e-8 || lk < 1e-8) return;
  double c = (rij[0] * rkj[0] + rij[1] * rkj[1] + rij[2] * rkj[2]) / (li * lk);
  c = fmax(-1.0, fmin(1.0, c));
  const double dth = acos(c) - (double)a->theta0;
  double sn = sqrt(1.0 - c * c);
  if (sn < 1e-8) sn = 1e-8;
  const double fm = -2.0 * (double)a->force_k * dth / sn;
  for (int d = 0; d < 3; ++d) {
    const double di = (rkj[d] / lk - c * rij[d] / li) / li;
    const double dk = (rij[d] / li - c * rkj[d] / lk) / lk;
    fi[d] -= fm * di;
    fk[d] -= fm * dk;
    fj[d] += fm * (di + dk);
  }
  *e += (double)a->force_k * dth * dth;
}

static void dihedral_f64(const double* x, const prismq_dihedral* t, double f0[3], double f1[3], double f2[3],
                         double f3[3], double* e) {
  double v0[3], v1[3], v2[3];
  for (int d = 0; d < 3; ++d) {
    v0[d] = x[3 * t->i + d] - x[3 * t->j + d];
    v1[d] = x[3 * t->k + d] - x[3 * t->j + d];
    v2[d] = x[3 * t->k + d] - x[3 * t->l + d];
  }
  const double c0[3] = {v0[1] * v1[2] - v0[2] * v1[1], v0[2] * v1[0] - v0[0] * v1[2], v0[0] * v1[1] - v0[1] * v1[0]};
  const double c1[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  const double n1 = c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2];
  const double n2 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
  const double nb = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
  if (n1 < 1e-16 || n2 < 1e-16 || nb < 1e-16) return;
  const double lbc = sqrt(nb);
  /* φ from atan2 (full precision in double) */
  const double xc[3] = {c0[1] * c1[2] - c0[2] * c1[1], c0[2] * c1[0] - c0[0] * c1[2], c0[0] * c1[1] - c0[1] * c1[0]};
  const double sn = sqrt(xc[0] * xc[0] + xc[1] * xc[1] + xc[2] * xc[2]);
  const double cs = c0[0] * c1[0] + c0[1] * c1[1] + c0[2] * c1[2];
  double phi = atan2(sn, cs);
  if (v0[0] * c1[0] + v0[1] * c1[1] + v0[2] * c1[2] < 0.0) phi = -phi;
  const double nn = (double)t->periodicity;
  const double dE = -(double)t->force_k * nn * sin(nn * phi - (double)t->phase);
  const double ff0 = (-dE * lbc) / n1;
  const double ff1 = (v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2]) / nb;
  const double ff2 = (v2[0] * v1[0] + v2[1] * v1[1] + v2[2] * v1[2]) / nb;
  const double ff3 = (dE * lbc) / n2;
  for (int d = 0; d < 3; ++d) {
    const double a1 = ff0 * c0[d], a4 = ff3 * c1[d];
    const double sv = ff1 * a1 - ff2 * a4;
    f0[d] += a1;
    f1[d] += sv - a1;
    f2[d] += -sv - a4;
    f3[d] += a4;
  }
  *e += (double)t->force_k * (1.0 + cos(nn * phi - (double)t->phase));
}

int orc_forces_f64(orc_sys* s, double* f, double* e5, int threads) {
  return orc_forces_f64_rule(s, f, e5, threads, 0);
}

/* incl64 = 0: ordinary pairs enter by the FP32 r^2 rule of the FP32 kernels
 * (the pair set the production path evaluates); incl64 = 1: by r^2 in double
 * (the pair set of the FP64-everywhere run). */
int orc_forces_f64_rule(orc_sys* s, double* f, double* e5, int threads, int incl64) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const int n = s->n;
  double* xd = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  for (int k = 0; k < 3 * n; ++k) xd[k] = (double)s->x[k];
  memset(f, 0, sizeof(double) * 3 * (size_t)n);
  double e[5] = {0, 0, 0, 0, 0};
  for (int t = 0; t < s->nb; ++t) {
    const prismq_bond* b = &s->bonds[t];
    bond_f64(xd, b, f + 3 * b->i, f + 3 * b->j, &e[0]);
  }
  for (int t = 0; t < s->na; ++t) {
    const prismq_angle* a = &s->angles[t];
    angle_f64(xd, a, f + 3 * a->i, f + 3 * a->j, f + 3 * a->k, &e[1]);
  }
  for (int t = 0; t < s->nd; ++t) {
    const prismq_dihedral* d = &s->dihs[t];
    dihedral_f64(xd, d, f + 3 * d->i, f + 3 * d->j, f + 3 * d->k, f + 3 * d->l, &e[2]);
  }
  /* exceptions, each pair once */
  for (int i = 0; i < n; ++i)
    for (int p = s->p14_off[i]; p < s->p14_off[i + 1]; ++p) {
      const int j = s->p14_j[p];
      if (j <= i) continue;
      double d[3];
      for (int c = 0; c < 3; ++c) d[c] = xd[3 * j + c] - xd[3 * i + c];
      const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (r2 < 1e-8) continue;
      const double inv_r = 1.0 / sqrt(r2), inv_r2 = inv_r * inv_r;
      const double sr2 = (double)s->p14_sig[p] * (double)s->p14_sig[p] * inv_r2;
      const double sr6 = sr2 * sr2 * sr2;
      const double eps = (double)s->p14_eps[p], qq = (double)s->p14_qq[p];
      const double fs = 24.0 * eps * inv_r2 * (2.0 * sr6 * sr6 - sr6) + (double)ORC_COULOMB * qq * inv_r2 * inv_r;
      for (int c = 0; c < 3; ++c) {
        f[3 * i + c] -= fs * d[c];
        f[3 * j + c] += fs * d[c];
      }
      e[3] += 4.0 * eps * (sr6 * sr6 - sr6) + (double)ORC_COULOMB * qq * inv_r;
    }
  /* ordinary pairs: candidates from a 10 Å grid over the current box, inclusion by
   * the FP32 rule, arithmetic in double */
  const float cut2 = s->p.cutoff * s->p.cutoff;
  const double rc = sqrt((double)cut2);
  orc_grid g;
  for (int d = 0; d < 3; ++d) {
    float lo = s->x[d], hi = s->x[d];
    for (int a = 1; a < n; ++a) {
      const float v = s->x[3 * a + d];
      if (v < lo) lo = v;
      if (v > hi) hi = v;
    }
    g.origin[d] = lo - ORC_CELL;
    g.dims[d] = (int)ceilf(((hi - lo) + 2.0f * ORC_CELL) / ORC_CELL);
  }
  int *start, *mem;
  cell_sort(n, s->x, &g, &start, &mem, NULL);
  double* fn = (double*)calloc(3 * (size_t)n, sizeof(double));
  double en = 0.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : en)
  for (int i = 0; i < n; ++i) {
    const int c = cell_of(&g, s->x + 3 * i);
    const int cx = c % g.dims[0], cy = (c / g.dims[0]) % g.dims[1], cz = c / (g.dims[0] * g.dims[1]);
    double fi[3] = {0, 0, 0};
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int X = cx + dx, Y = cy + dy, Z = cz + dz;
          if (X < 0 || Y < 0 || Z < 0 || X >= g.dims[0] || Y >= g.dims[1] || Z >= g.dims[2]) continue;
          const int cc = X + Y * g.dims[0] + Z * g.dims[0] * g.dims[1];
          for (int k = start[cc]; k < start[cc + 1]; ++k) {
            const int j = mem[k];
            if (j == i) continue;
            double d[3];
            for (int q = 0; q < 3; ++q) d[q] = xd[3 * j + q] - xd[3 * i + q];
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (incl64) {
              if (r2 >= (double)cut2 || r2 < (double)0.01f) continue;
            } else {
              float df[3];
              const float r2f = r2_force(s->x, i, j, df);
              if (r2f >= cut2 || r2f < 0.01f) continue;
            }
            if (excluded(i, j, s->all_off, s->all_list)) continue;
            const double inv_r = 1.0 / sqrt(r2), inv_r2 = inv_r * inv_r;
            const double sigma = 0.5 * ((double)s->sig[i] + (double)s->sig[j]);
            const double eps = sqrt((double)s->eps[i] * (double)s->eps[j]);
            const double qq = (double)s->q[i] * (double)s->q[j];
            const double sr2 = sigma * sigma * inv_r2, sr6 = sr2 * sr2 * sr2;
            const double fs = 24.0 * eps * inv_r2 * (2.0 * sr6 * sr6 - sr6) + (double)ORC_COULOMB * qq * inv_r2 * inv_r;
            for (int q = 0; q < 3; ++q) fi[q] -= fs * d[q];
            const double sc2 = sigma * sigma / (rc * rc), sc6 = sc2 * sc2 * sc2;
            const double v = 4.0 * eps * ((sr6 * sr6 - sr6) - (sc6 * sc6 - sc6)) +
                             (double)ORC_COULOMB * qq * (inv_r - 1.0 / rc);
            en += 0.5 * v;
          }
        }
    for (int q = 0; q < 3; ++q) fn[3 * i + q] = fi[q];
  }
  for (int k = 0; k < 3 * n; ++k) f[k] += fn[k];
  e[4] = en;
  free(fn);
  free(start);
  free(mem);
  free(xd);
  if (e5)
    for (int c = 0; c < 5; ++c) e5[c] = e[c];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Integrator phases, FP32 (nhs_amber_fused.cu:1713-2268, :3650-3831, :11128-11185). */
static void ou_atom(orc_sys* s, int a, long long step, uint32_t purpose) {
  if (s->p.gamma == 0.0f) return;
  const float c1 = s->p.c1;
  const float c2 = sqrtf((1.0f - c1 * c1) * ORC_AKMA * ORC_KB * s->p.temperature / s->m[a]);
  float z[3];
  orc_normal3(s->p.seed, s->p.stream, (uint32_t)a, (uint64_t)step, purpose, z);
  for (int d = 0; d < 3; ++d) s->v[3 * a + d] = c1 * s->v[3 * a + d] + c2 * z[d];
}

static void kick_atom(orc_sys* s, int a, const float* f) {
  const float kick = 0.5f * s->p.dt * ORC_AKMA / s->m[a];
  float* v = s->v + 3 * a;
  const float* F = f + 3 * a;
  if (s->p.gamma == 0.0f) {
    for (int d = 0; d < 3; ++d) v[d] += kick * F[d];
    return;
  }
  const float ax = F[0] * 1.0f, ay = F[1] * 1.0f, az = F[2] * 1.0f;
  const float mag = sqrtf(ax * ax + ay * ay + az * az);
  const float q = mag > ORC_MAXF ? ORC_MAXF / mag : 1.0f;
  v[0] = v[0] + kick * (ax * q);
  v[1] = v[1] + kick * (ay * q);
  v[2] = v[2] + kick * (az * q);
}

static int rattle_cluster(orc_sys* s, const orc_cluster* c) {
  const float tol = 1.0e-5f;
  float* x = s->x;
  float* v = s->v;
  const int ca = c->central;
  for (int it = 0; it < s->p.max_iter; ++it) {
    float maxe = 0.0f;
    for (int h = 0; h < c->nh; ++h) {
      const int ha = c->h[h];
      if (ha < 0) continue;
      const float rx = x[3 * ha] - x[3 * ca], ry = x[3 * ha + 1] - x[3 * ca + 1], rz = x[3 * ha + 2] - x[3 * ca + 2];
      const float r2 = rx * rx + ry * ry + rz * rz;
      if (!isfinite(r2) || r2 < 1.0e-12f) return 2;
      const float wx = v[3 * ha] - v[3 * ca], wy = v[3 * ha + 1] - v[3 * ca + 1], wz = v[3 * ha + 2] - v[3 * ca + 2];
      const float res = rx * wx + ry * wy + rz * wz;
      const float spd = sqrtf(wx * wx + wy * wy + wz * wz);
      const float scale = sqrtf(r2) * fmaxf(spd, 1.0f);
      const float rel = fabsf(res) / scale;
      if (!isfinite(rel)) return 2;
      maxe = fmaxf(maxe, rel);
      if (rel <= tol) continue;
      const float lam = res / ((c->imc + c->imh) * r2);
      const float cx = lam * rx, cy = lam * ry, cz = lam * rz;
      v[3 * ca] += c->imc * cx;
      v[3 * ca + 1] += c->imc * cy;
      v[3 * ca + 2] += c->imc * cz;
      v[3 * ha] -= c->imh * cx;
      v[3 * ha + 1] -= c->imh * cy;
      v[3 * ha + 2] -= c->imh * cz;
    }
    if (maxe <= tol) return 0;
  }
  return 2;
}

static int shake_cluster(orc_sys* s, const orc_cluster* c, const float* xs) {
  const float tol = 1.0e-4f;
  const float dt = s->p.dt;
  float* x = s->x;
  float* v = s->v;
  const int ca = c->central;
  for (int it = 0; it < s->p.max_iter; ++it) {
    float maxe = 0.0f;
    for (int h = 0; h < c->nh; ++h) {
      const int ha = c->h[h];
      if (ha < 0) continue;
      const float rx = x[3 * ha] - x[3 * ca], ry = x[3 * ha + 1] - x[3 * ca + 1], rz = x[3 * ha + 2] - x[3 * ca + 2];
      const float ox = xs[3 * ha] - xs[3 * ca], oy = xs[3 * ha + 1] - xs[3 * ca + 1], oz = xs[3 * ha + 2] - xs[3 * ca + 2];
      const float r2 = rx * rx + ry * ry + rz * rz;
      const float L = c->len[h];
      const float t2 = L * L;
      const float diff = r2 - t2;
      if (!isfinite(r2) || !isfinite(t2) || t2 <= 0.0f) return 1;
      const float rel = fabsf(diff) / t2;
      maxe = fmaxf(maxe, rel);
      if (rel <= tol) continue;
      const float rdo = rx * ox + ry * oy + rz * oz;
      const float o2 = ox * ox + oy * oy + oz * oz;
      const float ds = sqrtf(r2 * o2);
      if (!isfinite(rdo) || !isfinite(ds) || ds <= 0.0f || fabsf(rdo) / ds <= 1.0e-6f || !isfinite(dt) || dt <= 0.0f)
        return 1;
      const float lam = diff / (2.0f * (c->imc + c->imh) * rdo);
      const float cx = lam * ox, cy = lam * oy, cz = lam * oz;
      x[3 * ca] += c->imc * cx;
      x[3 * ca + 1] += c->imc * cy;
      x[3 * ca + 2] += c->imc * cz;
      x[3 * ha] -= c->imh * cx;
      x[3 * ha + 1] -= c->imh * cy;
      x[3 * ha + 2] -= c->imh * cz;
      v[3 * ca] += c->imc * cx / dt;
      v[3 * ca + 1] += c->imc * cy / dt;
      v[3 * ca + 2] += c->imc * cz / dt;
      v[3 * ha] -= c->imh * cx / dt;
      v[3 * ha + 1] -= c->imh * cy / dt;
      v[3 * ha + 2] -= c->imh * cz / dt;
    }
    if (maxe <= tol) return 0;
  }
  return 1;
}

static void clamp_atom(orc_sys* s, int a) {
  const float thermal = sqrtf(ORC_AKMA * ORC_KB * s->p.temperature / fmaxf(s->m[a], 1.0f));
  const float vmax = fmaxf(20.0f * thermal, 2.0f);
  float* v = s->v + 3 * a;
  const float mag = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (mag <= vmax) return;
  const float sc = vmax / mag;
  v[0] = v[0] * sc;
  v[1] = v[1] * sc;
  v[2] = v[2] * sc;
}

static int all_rattle(orc_sys* s) {
  int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
  for (int c = 0; c < s->ncl; ++c) err |= rattle_cluster(s, &s->cl[c]);
  return err;
}

static int phases_pre_f(orc_sys* s, const float* f, long long step, float* xs) {
  const int n = s->n;
  int err;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a) ou_atom(s, a, step, 1u);
  if ((err = all_rattle(s))) return err;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a) kick_atom(s, a, f);
  if ((err = all_rattle(s))) return err;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      xs[3 * a + d] = s->x[3 * a + d];
      s->x[3 * a + d] += s->p.dt * s->v[3 * a + d];
    }
  err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
  for (int c = 0; c < s->ncl; ++c) err |= shake_cluster(s, &s->cl[c], xs);
  return err;
}

static int phases_post_f(orc_sys* s, const float* f, long long step) {
  const int n = s->n;
  int err;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a) kick_atom(s, a, f);
  if ((err = all_rattle(s))) return err;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a) ou_atom(s, a, step, 2u);
#pragma omp parallel for schedule(static)
  for (int a = 0; a < n; ++a) clamp_atom(s, a);
  return all_rattle(s);
}

/* Single integrator pieces and per-term forces on the current state.  These
 * are the units the pins against the reference's own device functions
 * compare (tests/test_reference_kernels.py). */
int orc_rattle_all(orc_sys* s) { return all_rattle(s); }

int orc_shake_all(orc_sys* s, const float* xs) {
  int err = 0;
  for (int c = 0; c < s->ncl; ++c) err |= shake_cluster(s, &s->cl[c], xs);
  return err;
}

void orc_kick_all(orc_sys* s, const float* f) {
  for (int a = 0; a < s->n; ++a) kick_atom(s, a, f);
}

void orc_clamp_all(orc_sys* s) {
  for (int a = 0; a < s->n; ++a) clamp_atom(s, a);
}

/* One OU half-step of every atom with given normals z[3n] and a given c1,
 * the arithmetic of ou_atom (langevin_thermostat, nhs_amber_fused.cu:1713-1744). */
void orc_ou_all(orc_sys* s, const float* z, float c1) {
  if (s->p.gamma == 0.0f) return;
  for (int a = 0; a < s->n; ++a) {
    const float c2 = sqrtf((1.0f - c1 * c1) * ORC_AKMA * ORC_KB * s->p.temperature / s->m[a]);
    for (int d = 0; d < 3; ++d) s->v[3 * a + d] = c1 * s->v[3 * a + d] + c2 * z[3 * a + d];
  }
}

/* bonds -> fb[nb][2][3], angles -> fa[na][3][3], torsion terms -> fd[nd][4][3] */
void orc_term_forces(const orc_sys* s, float* fb, float* fa, float* fd) {
  for (int t = 0; t < s->nb; ++t) {
    float* o = fb + 6 * (size_t)t;
    for (int k = 0; k < 6; ++k) o[k] = 0.0f;
    bond_f32(s->x, &s->bonds[t], o, o + 3, NULL);
  }
  for (int t = 0; t < s->na; ++t) {
    float* o = fa + 9 * (size_t)t;
    for (int k = 0; k < 9; ++k) o[k] = 0.0f;
    angle_f32(s->x, &s->angles[t], o, o + 3, o + 6, NULL);
  }
  for (int t = 0; t < s->nd; ++t) {
    float* o = fd + 12 * (size_t)t;
    for (int k = 0; k < 12; ++k) o[k] = 0.0f;
    dihedral_f32(s->x, &s->dihs[t], o, o + 3, o + 6, o + 9, NULL);
  }
}

/* ---- run protocol (protocol_director.cu:54-143, fused_engine.rs:15366-15396) ----
 * e^x: x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r to degree 17 by
 * Horner's rule in binary64, times 2^k. */
static double orc_exp(double x) {
  if (x != x) return x;
  if (x < -708.0) return 0.0;
  if (x > 709.0) return HUGE_VAL;
  const double ln2 = 0.69314718055994530941723212145818;
  const double head = (double)(float)ln2, tail = ln2 - head;
  const double kd = floor(x / ln2 + 0.5);
  const double r = (x - kd * head) - kd * tail;
  double fact = 1.0, coef[18];
  for (int n = 0; n <= 17; ++n) {
    if (n > 0) fact *= (double)n;
    coef[n] = 1.0 / fact;
  }
  double p = coef[17];
  for (int n = 16; n >= 0; --n) p = p * r + coef[n];
  return ldexp(p, (int)kd);
}

void orc_protocol_eval(const prismq_protocol* P, long long director_step, float out[4]) {
  const int s = director_step > 2147483647LL ? 2147483647 : (int)director_step;
  const int e1 = P->cold_hold_steps, e2 = e1 + P->ramp_steps, e3 = e2 + P->warm_hold_steps,
            e4 = e3 + P->ramp_down_steps;
  float T;
  int hold;
  if (s < e1) {
    T = P->start_temp;
    hold = 1;
  } else if (s < e2) {
    const float prog = (float)(s - e1) / (float)(e2 - e1);
    T = P->start_temp + prog * (P->end_temp - P->start_temp);
    hold = 0;
  } else if (s < e3) {
    T = P->end_temp;
    hold = 1;
  } else if (s < e4) {
    const float prog = (float)(s - e3) / (float)(e4 - e3);
    T = P->end_temp - prog * (P->end_temp - P->start_temp);
    hold = 0;
  } else {
    T = (P->ramp_down_steps == 0 && P->cold_return_steps == 0) ? P->end_temp : P->start_temp;
    hold = 1;
  }
  float g = P->gamma_base;
  if (s < P->equilibration_steps) {
    const float prog = (float)s / (float)P->equilibration_steps;
    const float decay = (float)orc_exp((double)(-3.0f * prog));
    g = P->equilibration_gamma * decay + P->gamma_base * (1.0f - decay);
  }
  if (P->cryo_enabled && T < 300.0f) g = g * sqrtf(300.0f / (T > 10.0f ? T : 10.0f));
  float dt = P->base_dt;
  if (P->adaptive_dt == 2) dt = hold ? P->base_dt * 1.5f : P->base_dt;
  if (P->adaptive_dt == 1) dt = hold ? P->base_dt : P->base_dt * 0.5f;
  out[0] = T;
  out[1] = g;
  out[2] = dt;
  out[3] = (float)orc_exp((double)(-g * (0.5f * dt)));
}

void orc_set_protocol(orc_sys* s, const prismq_protocol* p, long long origin) {
  s->proto_on = p != NULL;
  if (p) s->proto = *p;
  s->proto_origin = origin;
}

/* The parameters of step `step` under the installed protocol. */
static void protocol_step(orc_sys* s, long long step) {
  if (!s->proto_on) return;
  float o[4];
  orc_protocol_eval(&s->proto, step - s->proto_origin, o);
  s->p.temperature = o[0];
  s->p.gamma = o[1];
  s->p.dt = o[2];
  s->p.c1 = o[3];
}

int orc_phases(orc_sys* s, int set, const int64_t* f_fixed, long long step) {
  protocol_step(s, step);
  const int n = s->n;
  float* f = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  for (int k = 0; k < 3 * n; ++k) f[k] = orc_fixed2f(f_fixed[k]);
  int err;
  if (set == 1) {
    float* xs = (float*)malloc(sizeof(float) * 3 * (size_t)n);
    err = phases_pre_f(s, f, step, xs);
    free(xs);
  } else {
    err = phases_post_f(s, f, step);
  }
  free(f);
  return err;
}

/* COM velocity removal (housekeeping.cu:128-183): Σ m·v, Σ m, v -= Σmv/Σm.
 * Σ m·v in exact int64 fixed point and Σ m in double make it order-free. */
void orc_com_remove(orc_sys* s) {
  int64_t P[3] = {0, 0, 0};
  double M = 0.0;
  for (int a = 0; a < s->n; ++a) {
    for (int d = 0; d < 3; ++d) P[d] += orc_f2fixed(s->m[a] * s->v[3 * a + d]);
    M += (double)s->m[a];
  }
  float vc[3] = {0, 0, 0};
  if (M > 0.0)
    for (int d = 0; d < 3; ++d) vc[d] = (float)((double)P[d] * 2.3283064365386963e-10 / M);
  for (int a = 0; a < s->n; ++a)
    for (int d = 0; d < 3; ++d) s->v[3 * a + d] = s->v[3 * a + d] - vc[d];
}

/* Reference step loop: MD_EXECUTION_PHASES (fused_engine.rs:6223-6235), rebuild at
 * step start every 20 steps (:19106-19125) and after every SHAKE (:19441-19455),
 * COM removal at step start every com_interval steps (:19010-19075). */
int orc_run(orc_sys* s, long n_steps, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const int n = s->n;
  float* f = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  float* xs = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  int err = 0;
  for (long it = 0; it < n_steps && !err; ++it) {
    const long long st = s->step;
    protocol_step(s, st);
    if (s->p.com_interval > 0 && st > 0 && st % s->p.com_interval == 0) orc_com_remove(s);
    const int rebuild = (st == 0) || (st % 20 == 0);
    if ((err = forces_f32_impl(s, f, NULL, rebuild))) break;     /* FORCE_N */
    if ((err = phases_pre_f(s, f, st, xs))) break;                /* 10,11,12,2,3,4 */
    if ((err = forces_f32_impl(s, f, NULL, 1))) break;            /* rebuild + FORCE_NP1 */
    if ((err = phases_post_f(s, f, st))) break;                   /* 13,14,15, clamp, RATTLE */
    s->step = st + 1;
  }
  free(f);
  free(xs);
  return err;
}
