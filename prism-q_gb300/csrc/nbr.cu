// Per-system step control, cell lists and neighbour rows (compiled with --fmad=false).
//
// Reference path (nhs_amber_fused.cu:11690-11790, nhs_neighbor_warp.cuh:10-121,
// fused_engine.rs:16615-16700): a fixed 10 Å grid from the construction-time
// bounding box, cell slots claimed by atomicAdd, a warp-per-atom 27-cell scan
// with r^2 <= (1.2·cutoff)^2, exclusion scan, and a per-row bitonic sort,
// rebuilt every step.
//
// GB300 form:
//   k_control_cells  one CTA per system: COM removal + deferred pre-phase on
//                    COM steps, rebuild decision (interval or half-skin
//                    displacement), bounding box, counting sort of atoms into
//                    cells and an ascending sort of each cell's contents, so
//                    that rows come out in a deterministic order without a
//                    per-row sort.  It then queues the 8-atom groups of every
//                    rebuilding system on a device work list.
//   k_nbr_build      one warp per queued 8-atom group at a time (a grid of
//                    the resident CTAs; round-robin over the queue when it
//                    runs beside the forces of a many-system step, from a
//                    shared counter when it runs alone).  The warp lists the
//                    cell-row runs of the union of its atoms' stencils (the
//                    x-run of cells in one (y, z) row is one contiguous run
//                    of sorted atoms), streams
//                    their candidates in full 32-lane chunks, tests each
//                    against the eight atoms, applies the exclusion window
//                    bitmask and ballot-compacts the kept atoms straight into
//                    the tiled layout the force kernel reads.  REF27 rows are
//                    built atom by atom with the reference's stencil.  Steps
//                    without rebuilds cost one empty pass.
// Complete mode uses cells at least r_list/2 wide with a ±2 stencil (every
// pair within r_list is found); REF27 mode reproduces the reference pair set.
#include <algorithm>

#include "pq_phases.cuh"

namespace pq {

// r^2 in the reference's uncontracted FP32 order: (dx*dx + dy*dy) + dz*dz,
// the order scripts/physics_refs/neighbor_list.py:63-91 evaluates.
__device__ __forceinline__ float r2_nofma(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

constexpr int kCtlThreads = 1024;
constexpr int kCellSortCap = 512;  // per-cell sort scratch (and overflow bound)

__device__ __forceinline__ int cell_coord(float x, float lo, float inv_edge, int n) {
  int c = (int)((x - lo) * inv_edge);
  return c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
}

// The cell of a position on the system's current grid.
__device__ __forceinline__ int cell_of(const float4 p, int nbr_mode, const float (&lo)[3], const float (&inv_edge)[3],
                                       const int (&dims)[3]) {
  int ix, iy, iz;
  if (nbr_mode == 1) {
    // reference rule: truncate (x - origin) * 0.1f toward zero, then clamp
    ix = (int)((p.x - lo[0]) * 0.1f);
    iy = (int)((p.y - lo[1]) * 0.1f);
    iz = (int)((p.z - lo[2]) * 0.1f);
    ix = max(0, min(ix, dims[0] - 1));
    iy = max(0, min(iy, dims[1] - 1));
    iz = max(0, min(iz, dims[2] - 1));
  } else {
    ix = cell_coord(p.x, lo[0], inv_edge[0], dims[0]);
    iy = cell_coord(p.y, lo[1], inv_edge[1], dims[1]);
    iz = cell_coord(p.z, lo[2], inv_edge[2], dims[2]);
  }
  return ix + iy * dims[0] + iz * dims[0] * dims[1];
}

// The grid a system's last control pass chose (REF27: the fixed reference grid).
__device__ __forceinline__ void grid_of(const SysDev* Sp, float (&lo)[3], float (&inv_edge)[3], int (&dims)[3]) {
  for (int d = 0; d < 3; ++d) {
    if (Sp->nbr_mode == 1) {
      lo[d] = Sp->ref_origin[d];
      inv_edge[d] = 0.1f;
      dims[d] = Sp->ref_dims[d];
    } else {
      lo[d] = Sp->g_lo[d];
      inv_edge[d] = Sp->g_inv_edge[d];
      dims[d] = Sp->g_dims[d];
    }
  }
}

// Ascending order of one cell's atoms, by one warp (bitonic in its scratch).
__device__ __forceinline__ void sort_cell(int* cell, int n, int* buf, int lane) {
  if (n <= 1) return;
  int p2 = 1;
  while (p2 < n) p2 <<= 1;
  for (int k = lane; k < p2; k += 32) buf[k] = k < n ? cell[k] : 0x7fffffff;
  __syncwarp();
  for (int w = 2; w <= p2; w <<= 1) {
    for (int st = w >> 1; st > 0; st >>= 1) {
      for (int k = lane; k < p2; k += 32) {
        const int q = k ^ st;
        if (q > k) {
          const int x = buf[k], y = buf[q];
          const bool up = (k & w) == 0;
          if ((up && x > y) || (!up && x < y)) {
            buf[k] = y;
            buf[q] = x;
          }
        }
      }
      __syncwarp();
    }
  }
  for (int k = lane; k < n; k += 32) cell[k] = buf[k];
  __syncwarp();
}

// COM-velocity removal of one system followed by its deferred pre-phase
// (every com_interval steps; housekeeping.cu:128-183 reduces with FP32
// atomics).  FP32 systems sum m·v as exact int64 fixed point and m exactly in
// double; FP64 systems sum in double.  Both reductions use a fixed order, so
// the result does not depend on scheduling.
template <class R, bool kCheck64>
__device__ __noinline__ void com_pre(const Arena& A, SysDev* Sp, long long st, long long (*red_i)[32], double (*red)[32],
                        double* sh_vcom) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ab = Sp->atom_begin, na = Sp->n_atoms;
  long long px = 0, py = 0, pz = 0;
  double qx = 0.0, qy = 0.0, qz = 0.0, m = 0.0;
  for (int i = tid; i < na; i += kCtlThreads) {
    if (sizeof(R) == 4) {
      const float4 v = A.vel[ab + i];
      px += f2fixed(v.w * v.x);
      py += f2fixed(v.w * v.y);
      pz += f2fixed(v.w * v.z);
      m += (double)v.w;
    } else {
      const double4_32a v = A.vel64[ab + i];
      qx += v.w * v.x;
      qy += v.w * v.y;
      qz += v.w * v.z;
      m += v.w;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    px += __shfl_xor_sync(0xffffffffu, px, o);
    py += __shfl_xor_sync(0xffffffffu, py, o);
    pz += __shfl_xor_sync(0xffffffffu, pz, o);
    qx += __shfl_xor_sync(0xffffffffu, qx, o);
    qy += __shfl_xor_sync(0xffffffffu, qy, o);
    qz += __shfl_xor_sync(0xffffffffu, qz, o);
    m += __shfl_xor_sync(0xffffffffu, m, o);
  }
  if (lane == 0) {
    red_i[0][warp] = px;
    red_i[1][warp] = py;
    red_i[2][warp] = pz;
    red[0][warp] = qx;
    red[1][warp] = qy;
    red[2][warp] = qz;
    red[3][warp] = m;
  }
  __syncthreads();
  if (tid == 0) {
    long long IX = 0, IY = 0, IZ = 0;
    double X = 0.0, Y = 0.0, Z = 0.0, M = 0.0;
    for (int w = 0; w < 32; ++w) {
      IX += red_i[0][w];
      IY += red_i[1][w];
      IZ += red_i[2][w];
      X += red[0][w];
      Y += red[1][w];
      Z += red[2][w];
      M += red[3][w];
    }
    double c[3] = {0.0, 0.0, 0.0};
    if (M > 0.0) {
      if (sizeof(R) == 4) {
        // the FP32 systems subtract the float COM velocity
        c[0] = (double)(float)((double)IX * kFixedInvD / M);
        c[1] = (double)(float)((double)IY * kFixedInvD / M);
        c[2] = (double)(float)((double)IZ * kFixedInvD / M);
      } else {
        c[0] = X / M;
        c[1] = Y / M;
        c[2] = Z / M;
      }
    }
    for (int d = 0; d < 3; ++d) {
      sh_vcom[d] = c[d];
      Sp->vcom[d] = c[d];
    }
  }
  __syncthreads();
  const SysDev S = *Sp;
  for (int t = tid; t < S.n_units; t += kCtlThreads) {
    const Unit U = A.units[S.unit_begin + t];
    if (U.nh < 0) continue;
    UnitStateT<R> u;
    int local[4];
    load_unit(A, U, u, local, ab);
    for (int k = 0; k < u.n; ++k) {
      u.vx[k] = u.vx[k] - R(sh_vcom[0]);
      u.vy[k] = u.vy[k] - R(sh_vcom[1]);
      u.vz[k] = u.vz[k] - R(sh_vcom[2]);
    }
    int err = phases_pre<R, kCheck64>(u, U, S, local, (uint64_t)st);
    if (!err && !unit_finite(u)) err = kStNonfinite;
    if (err) {
      atomicOr(&Sp->status, err);
      continue;
    }
    check_displacement(A, U, u, Sp);
    store_unit(A, U, u, true);
  }
  __syncthreads();
}

// The schedule decision of one step: rebuild the list or not (interval or
// half-skin displacement), advance the step counter, keep this step's
// parameters for its post-force phases and, under a protocol, evaluate the
// director for the next step's pre-force phases (protocol_director.cu:54-143).
__device__ bool decide_step(SysDev* Sp, int disp, int status) {
  bool rb = !Sp->built || disp || Sp->steps_since_rebuild >= Sp->rebuild_interval;
  Sp->step = Sp->step + 1;
  Sp->post_dt = Sp->dt;
  Sp->post_temperature = Sp->temperature;
  Sp->post_gamma = Sp->gamma;
  Sp->post_c1 = Sp->c1;
  Sp->post_c1d = Sp->c1d;
  if (Sp->proto.on) {
    StepParams P;
    protocol_eval(Sp->proto, Sp->step - Sp->proto.origin, &P);
    Sp->dt = P.dt;
    Sp->temperature = P.temperature;
    Sp->gamma = P.gamma;
    Sp->c1 = P.c1;
    Sp->c1d = P.c1d;
  }
  if (status != 0) rb = false;
  Sp->steps_since_rebuild = rb ? 1 : Sp->steps_since_rebuild + 1;
  Sp->displaced = 0;
  Sp->rebuilding = rb ? 1 : 0;
  if (rb) Sp->n_rebuilds += 1;
  return rb;
}

// One thread per system at the start of every step.  Systems at a COM step
// are left to the control kernel, which removes the COM velocity and runs
// their deferred pre-force phases before it decides.
__global__ void __launch_bounds__(128) k_decide(Arena A, int n_sys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sys) return;
  SysDev* Sp = &A.sys[s];
  if (!Sp->active) return;
  if (Sp->status != 0) {
    Sp->branch_a = 0;
    return;
  }
  const long long st = Sp->step;
  if (Sp->com_interval > 0 && st > 0 && (st % Sp->com_interval) == 0) {
    Sp->com_pending = 1;
    Sp->branch_a = 1;
    return;
  }
  Sp->com_pending = 0;
  Sp->branch_a = decide_step(Sp, Sp->displaced, 0) ? 1 : 0;
}

void launch_decide(const Arena& A, int n_sys, cudaStream_t st) {
  if (n_sys <= 0) return;
  k_decide<<<(n_sys + 127) / 128, 128, 0, st>>>(A, n_sys);
}

__global__ void __launch_bounds__(kCtlThreads) k_control_cells(Arena A, int mode, int nbr_override) {
  extern __shared__ int sm[];  // per-warp sort scratch: 32 * kCellSortCap ints
  __shared__ long long red_i[3][32];
  __shared__ double red_d[4][32];
  __shared__ float red_f[6][32];
  __shared__ int sh_rb;
  __shared__ double sh_vcomd[3];
  const int s = blockIdx.x;
  SysDev* Sp = &A.sys[s];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (!Sp->active) return;
  if (Sp->status != 0) return;
  const int ab = Sp->atom_begin, na = Sp->n_atoms;
  // in a step, k_decide has already decided for every system not at a COM step
  const bool decided = mode == kCtlStep && !Sp->com_pending;
  if (decided && !Sp->rebuilding) return;

  if (mode == kCtlStep && !decided) {
    const long long st = Sp->step;
    {
      if (A.fp64)
        com_pre<double, false>(A, Sp, st, red_i, red_d, sh_vcomd);
      else if (Sp->check64)
        com_pre<float, true>(A, Sp, st, red_i, red_d, sh_vcomd);
      else
        com_pre<float, false>(A, Sp, st, red_i, red_d, sh_vcomd);
    }
  }

  if (tid == 0) {
    bool rb;
    if (decided) {
      rb = true;  // k_decide chose a rebuild
    } else if (mode == kCtlStep) {
      // a COM step: decide after the pre-force phases ran above
      rb = decide_step(Sp, atomicAdd(&Sp->displaced, 0), atomicAdd(&Sp->status, 0));
      Sp->com_pending = 0;
    } else {
      if (mode == kCtlPrime) {
        rb = Sp->need_prime != 0;
        Sp->need_prime = 0;
      } else {
        rb = true;
      }
      if (atomicAdd(&Sp->status, 0) != 0) rb = false;
      // A prime pass (another system was admitted or reset) leaves the
      // schedule of the systems it does not rebuild untouched, so a system's
      // trajectory never depends on what else shares the batch.
      if (mode != kCtlPrime || rb) {
        Sp->steps_since_rebuild = rb ? 1 : Sp->steps_since_rebuild + 1;
        Sp->displaced = 0;
      }
      Sp->rebuilding = rb ? 1 : 0;
      if (rb) Sp->n_rebuilds += 1;
      if (nbr_override >= 0 && rb) Sp->nbr_mode = nbr_override;
    }
    sh_rb = rb ? 1 : 0;
  }
  __syncthreads();
  if (!sh_rb) return;

  // ---- grid ----
  const int nbr_mode = Sp->nbr_mode;
  float lo[3], inv_edge[3];
  int dims[3];
  if (nbr_mode == 1) {
    for (int d = 0; d < 3; ++d) {
      lo[d] = Sp->ref_origin[d];
      inv_edge[d] = 0.1f;
      dims[d] = Sp->ref_dims[d];
    }
  } else {
    float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int i = tid; i < na; i += kCtlThreads) {
      const float4 p = A.pos[ab + i];
      mn[0] = fminf(mn[0], p.x);
      mn[1] = fminf(mn[1], p.y);
      mn[2] = fminf(mn[2], p.z);
      mx[0] = fmaxf(mx[0], p.x);
      mx[1] = fmaxf(mx[1], p.y);
      mx[2] = fmaxf(mx[2], p.z);
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int d = 0; d < 3; ++d) {
        mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
        mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
      }
    if (lane == 0)
      for (int d = 0; d < 3; ++d) {
        red_f[d][warp] = mn[d];
        red_f[3 + d][warp] = mx[d];
      }
    __syncthreads();
    if (tid == 0) {
      float gl[3], gh[3];
      for (int d = 0; d < 3; ++d) {
        gl[d] = red_f[d][0];
        gh[d] = red_f[3 + d][0];
        for (int w = 1; w < 32; ++w) {
          gl[d] = fminf(gl[d], red_f[d][w]);
          gh[d] = fmaxf(gh[d], red_f[3 + d][w]);
        }
      }
      // cells at least r_list/2·(1+1e-4) wide on every axis; the row builder
      // scans ±2 cells, which covers every pair within r_list
      // (y and z; x cells are only r_list/4 wide because rows are scanned as
      // contiguous x-runs trimmed per atom to the sphere of radius r_list)
      const float edge_yz = sqrtf(Sp->rlist2) * 0.50005f;
      int nd[3];
      float ext[3];
      for (int d = 0; d < 3; ++d) {
        ext[d] = fmaxf(gh[d] - gl[d], 1.0e-3f);
        const float q = ext[d] / (d == 0 ? 0.5f * edge_yz : edge_yz);
        nd[d] = q >= 1.0f ? (int)q : 1;
        if (nd[d] > 1024) nd[d] = 1024;
      }
      while ((long long)nd[0] * nd[1] * nd[2] > Sp->cell_cap) {
        int big = 0;
        if (nd[1] > nd[big]) big = 1;
        if (nd[2] > nd[big]) big = 2;
        nd[big] -= 1;
      }
      for (int d = 0; d < 3; ++d) {
        Sp->g_lo[d] = gl[d];
        Sp->g_dims[d] = nd[d];
        Sp->g_inv_edge[d] = (float)nd[d] / ext[d];
      }
    }
    __syncthreads();
    for (int d = 0; d < 3; ++d) {
      lo[d] = Sp->g_lo[d];
      inv_edge[d] = Sp->g_inv_edge[d];
      dims[d] = Sp->g_dims[d];
    }
  }
  const int ncell = dims[0] * dims[1] * dims[2];
  int* start = A.cell_start + Sp->cell_begin;     // ncell + 1 entries
  int* cursor = start + (Sp->cell_cap + 1);       // ncell entries

  // ---- counting sort ----
  for (int c = tid; c <= ncell; c += kCtlThreads) start[c] = 0;
  __syncthreads();
  if (na >= kBigSortAtoms) {
    // a large system: the grid-wide kernels that follow sort its cells
    __shared__ int sh_base_big;
    const int ngroups = (na + 7) >> 3;
    if (tid == 0) {
      Sp->built = 1;
      A.big_list[atomicAdd(&A.work_ctl[1], 1)] = s;
      sh_base_big = atomicAdd(&A.work_ctl[0], ngroups);
    }
    __syncthreads();
    for (int i = tid; i < ngroups; i += kCtlThreads) A.work[sh_base_big + i] = (ab >> 3) + i;
    return;
  }
  for (int i = tid; i < na; i += kCtlThreads) {
    const int a = ab + i;
    const int c = cell_of(A.pos[a], nbr_mode, lo, inv_edge, dims);
    A.atom_cell[a] = c;
    atomicAdd(&start[c + 1], 1);
  }
  __syncthreads();
  // exclusive scan (single-thread prefix over warp partials)
  {
    __shared__ int wsum[32];
    __shared__ int carry;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ncell; base += kCtlThreads) {
      const int c = base + tid;
      int v = c < ncell ? start[c + 1] : 0;
      if (v > kCellSortCap) atomicOr(&Sp->status, kStCellOverflow);
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) wsum[warp] = x;
      __syncthreads();
      if (warp == 0) {
        int w = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += y;
        }
        wsum[lane] = w;
      }
      __syncthreads();
      const int incl = x + (warp > 0 ? wsum[warp - 1] : 0) + carry;
      if (c < ncell) {
        start[c + 1] = incl;
        cursor[c] = incl - v;
      }
      __syncthreads();
      if (tid == kCtlThreads - 1) carry = incl;
      __syncthreads();
    }
  }
  if (atomicAdd(&Sp->status, 0) != 0) return;
  for (int i = tid; i < na; i += kCtlThreads) {
    const int a = ab + i;
    const int c = A.atom_cell[a];
    const int slot = atomicAdd(&cursor[c], 1);
    A.cell_atoms[ab + slot] = a;
  }
  __syncthreads();
  // ---- ascending order inside each cell (warp per cell, bitonic in smem) ----
  int* buf = sm + warp * kCellSortCap;
  for (int c = warp; c < ncell; c += kCtlThreads / 32) {
    const int b = start[c];
    sort_cell(A.cell_atoms + ab + b, start[c + 1] - b, buf, lane);
  }
  // queue this system's 8-atom groups for the row builder
  __shared__ int sh_base;
  const int ngroups = (na + 7) >> 3;  // 8-atom work items
  if (tid == 0) {
    Sp->built = 1;
    sh_base = atomicAdd(&A.work_ctl[0], ngroups);
  }
  __syncthreads();
  for (int i = tid; i < ngroups; i += kCtlThreads) A.work[sh_base + i] = (ab >> 3) + i;
}

// Persistent row builder: resident CTAs of eight warps pull 8-atom groups of
// rebuilding systems from the work list and write each kept neighbour
// straight into the tiled layout.
constexpr int kNbrThreads = 256;

__device__ __forceinline__ void build_row(const Arena& A, int a, int exclude_exc, int lane, int* count_out) {
  int count = -1;
  const int s = A.atom_sys[a];
  SysDev* Sp = s >= 0 ? &A.sys[s] : nullptr;
  if (Sp && Sp->active && Sp->rebuilding && Sp->status == 0) {
    const int ab = Sp->atom_begin;
    const int mode = Sp->nbr_mode;
    int dims[3];
    if (mode == 1) {
      dims[0] = Sp->ref_dims[0];
      dims[1] = Sp->ref_dims[1];
      dims[2] = Sp->ref_dims[2];
    } else {
      dims[0] = Sp->g_dims[0];
      dims[1] = Sp->g_dims[1];
      dims[2] = Sp->g_dims[2];
    }
    const float r2max = mode == 1 ? Sp->ref_r2 : Sp->rlist2;
    const int* start = A.cell_start + Sp->cell_begin;
    const float4 pi = A.pos[a];
    const int cell = A.atom_cell[a];
    const int cx = cell % dims[0], cy = (cell / dims[0]) % dims[1], cz = cell / (dims[0] * dims[1]);
    const unsigned long long mask = exclude_exc ? A.mask_all[a] : A.mask_ref[a];
    const int2 far = A.far[a];
    // REF27: the reference's 27 cells of 10 Å.  Complete: rows of y/z cells
    // (>= r_list/2 wide) within ±2, each scanned over the x-range that can hold
    // atoms within r_list of atom a.  The trimming is conservative (cell
    // indices are monotone in the coordinate, slab distances carry a 1e-3 Å
    // margin), so it only removes candidates the r^2 test would reject.
    const int reach = mode == 1 ? 1 : 2;
    const float lox = Sp->g_lo[0], loy = Sp->g_lo[1], loz = Sp->g_lo[2];
    const float ivx = Sp->g_inv_edge[0];
    const float ey = 1.0f / Sp->g_inv_edge[1], ez = 1.0f / Sp->g_inv_edge[2];
    count = 0;
    bool overflow = false;
    for (int dz = -reach; dz <= reach; ++dz) {
      const int z = cz + dz;
      if (z < 0 || z >= dims[2]) continue;
      for (int dy = -reach; dy <= reach; ++dy) {
        const int y = cy + dy;
        if (y < 0 || y >= dims[1]) continue;
        int x0, x1;
        if (mode == 1) {
          x0 = max(cx - 1, 0);
          x1 = min(cx + 1, dims[0] - 1);
        } else {
          const float sy = fmaxf(0.0f, fmaxf((loy + (float)y * ey) - pi.y, pi.y - (loy + (float)(y + 1) * ey)));
          const float sz = fmaxf(0.0f, fmaxf((loz + (float)z * ez) - pi.z, pi.z - (loz + (float)(z + 1) * ez)));
          const float my = fmaxf(sy - 1.0e-3f, 0.0f), mz = fmaxf(sz - 1.0e-3f, 0.0f);
          const float d2 = my * my + mz * mz;
          if (d2 > r2max) continue;
          const float xr = sqrtf(r2max - d2) + 1.0e-3f;
          x0 = max((int)((pi.x - xr - lox) * ivx), 0);
          x1 = min((int)((pi.x + xr - lox) * ivx), dims[0] - 1);
          if (x0 > x1) continue;
        }
        // the x-run of cells in one (y, z) row is one contiguous run of atoms
        const int rowc = y * dims[0] + z * dims[0] * dims[1];
        const int b = start[rowc + x0], e = start[rowc + x1 + 1];
        for (int base = b; base < e; base += 32) {
          const int k = base + lane;
          int j = 0;
          bool keep = false;
          if (k < e) {
            j = A.cell_atoms[ab + k];
            if (j != a) {
              const float4 pj = A.pos[j];
              const float r2 = r2_nofma(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z);
              keep = !(r2 > r2max);
              if (keep) {
                const int d = j - a;
                if (d >= -32 && d < 32) {
                  if ((mask >> (d + 32)) & 1ull) keep = false;
                } else {
                  for (int q = 0; q < far.y; ++q) {
                    const int ent = A.far_list[far.x + q];
                    if ((ent & 0x3fffffff) == j && (exclude_exc || !(ent & 0x40000000))) {
                      keep = false;
                      break;
                    }
                  }
                }
              }
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, keep);
          const int add = __popc(bal);
          if (count + add > kNbrCap) {
            overflow = true;
          } else {
            if (keep) A.nbr[nbr_index(a, count + __popc(bal & ((1u << lane) - 1u)))] = j;
            count += add;
          }
        }
      }
    }
    if (overflow) {
      if (lane == 0) atomicOr(&Sp->status, kStNbrOverflow);
      count = -1;
    } else if (lane == 0) {
      A.nnbr[a] = count;
      A.xref[a] = pi;
    }
  }
  *count_out = count;
}

// Per-warp data of the group being built: the atoms' exclusion data and the
// candidate runs (one per cell row of the union stencil, in (z, y) order).
constexpr int kMaxRuns = 96;
struct GroupShared {
  unsigned long long mask[8];
  int2 far[8];
  int run_b[kMaxRuns];        // first sorted-atom index of the run
  int run_off[kMaxRuns + 1];  // exclusive prefix of run lengths
  // cluster-pair tiles of the group: open-addressing table keyed by the
  // system-local j-cluster + 1 (0 = empty), with the OR of its pair bits.
  // The table lives after the warps' GroupShared records and only in
  // launches for the tile layout (kTileHash keys and masks per warp).
  int* tkey;
  unsigned* tmask;
  int tcount;  // keys in the table
};
constexpr size_t kTileTableBytes = (size_t)kTileHash * (sizeof(int) + sizeof(unsigned));

// Add pair bits to j-cluster jc_local's entry of the group's tile table.  The
// table's contents (a set of keys with OR-ed masks) do not depend on the order
// of insertion.  Returns false once the group holds more than kTileCap
// j-clusters (the table then stays at most 3/4 full, so probes stay short).
__device__ __forceinline__ bool tile_insert(GroupShared& sh, int jc_local, unsigned bits) {
  if (*(volatile int*)&sh.tcount > kTileCap) return false;
  const int key = jc_local + 1;
  unsigned h = ((unsigned)key * 2654435761u) >> 22;  // top 10 bits: kTileHash = 1024 slots
  for (int probe = 0; probe < kTileHash; ++probe) {
    const int prev = atomicCAS(&sh.tkey[h], 0, key);
    if (prev == 0 || prev == key) {
      atomicOr(&sh.tmask[h], bits);
      return prev == key || atomicAdd(&sh.tcount, 1) < kTileCap;
    }
    h = (h + 1) & (kTileHash - 1);
  }
  return false;
}

// The group's tiles out of its table: compacted, sorted by j-cluster (so the
// list order is a function of the pair set alone) and written as
// {global j-cluster, mask}.  Returns the tile count, or -1 past kTileCap.
__device__ int tile_flush(const Arena& A, GroupShared& sh, int64_t g, int ab, int lane) {
  __syncwarp();
  int cnt = 0;
  for (int b = 0; b < kTileHash; b += 32) {
    const int k = sh.tkey[b + lane];
    const unsigned m = sh.tmask[b + lane];
    const unsigned bal = __ballot_sync(0xffffffffu, k != 0);
    __syncwarp();
    if (k != 0) {
      const int at = cnt + __popc(bal & ((1u << lane) - 1u));
      sh.tkey[at] = k;
      sh.tmask[at] = m;
    }
    cnt += __popc(bal);
    __syncwarp();
  }
  if (cnt > kTileCap) return -1;
  int p2 = 1;
  while (p2 < cnt) p2 <<= 1;
  for (int k = cnt + lane; k < p2; k += 32) sh.tkey[k] = 0x7fffffff;
  __syncwarp();
  for (int w = 2; w <= p2; w <<= 1)
    for (int st = w >> 1; st > 0; st >>= 1) {
      for (int k = lane; k < p2; k += 32) {
        const int q = k ^ st;
        if (q > k) {
          const int x = sh.tkey[k], y = sh.tkey[q];
          const bool up = (k & w) == 0;
          if ((up && x > y) || (!up && x < y)) {
            sh.tkey[k] = y;
            sh.tkey[q] = x;
            const unsigned mx = sh.tmask[k];
            sh.tmask[k] = sh.tmask[q];
            sh.tmask[q] = mx;
          }
        }
      }
      __syncwarp();
    }
  int2* out = A.tiles + g * kTileCap;
  for (int k = lane; k < cnt; k += 32) out[k] = make_int2((ab >> 2) + sh.tkey[k] - 1, (int)sh.tmask[k]);
  if (lane == 0) A.ntile[g] = cnt;
  __syncwarp();
  return cnt;
}

// Tiles input of one atom (i of the group) from its own stencil, as
// build_row scans it: used for a group whose union stencil is too large.
__device__ bool tile_atom(const Arena& A, const SysDev* Sp, GroupShared& sh, int a, int i, int lane,
                          int exclude_exc) {
  const int ab = Sp->atom_begin;
  const int dims[3] = {Sp->g_dims[0], Sp->g_dims[1], Sp->g_dims[2]};
  const float r2max = Sp->rlist2;
  const int* start = A.cell_start + Sp->cell_begin;
  const float4 pi = A.pos[a];
  const int cell = A.atom_cell[a];
  const int cx = cell % dims[0], cy = (cell / dims[0]) % dims[1], cz = cell / (dims[0] * dims[1]);
  const unsigned long long mask = exclude_exc ? A.mask_all[a] : A.mask_ref[a];
  const int2 far = A.far[a];
  const float lox = Sp->g_lo[0], loy = Sp->g_lo[1], loz = Sp->g_lo[2];
  const float ivx = Sp->g_inv_edge[0];
  const float ey = 1.0f / Sp->g_inv_edge[1], ez = 1.0f / Sp->g_inv_edge[2];
  bool ok = true;
  for (int dz = -2; dz <= 2; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= dims[2]) continue;
    for (int dy = -2; dy <= 2; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= dims[1]) continue;
      const float sy = fmaxf(0.0f, fmaxf((loy + (float)y * ey) - pi.y, pi.y - (loy + (float)(y + 1) * ey)));
      const float sz = fmaxf(0.0f, fmaxf((loz + (float)z * ez) - pi.z, pi.z - (loz + (float)(z + 1) * ez)));
      const float my = fmaxf(sy - 1.0e-3f, 0.0f), mz = fmaxf(sz - 1.0e-3f, 0.0f);
      const float d2 = my * my + mz * mz;
      if (d2 > r2max) continue;
      const float xr = sqrtf(r2max - d2) + 1.0e-3f;
      const int x0 = max((int)((pi.x - xr - lox) * ivx), 0);
      const int x1 = min((int)((pi.x + xr - lox) * ivx), dims[0] - 1);
      if (x0 > x1) continue;
      const int rowc = y * dims[0] + z * dims[0] * dims[1];
      const int b = start[rowc + x0], e = start[rowc + x1 + 1];
      for (int base = b; base < e; base += 32) {
        const int k = base + lane;
        if (k >= e) continue;
        const int j = A.cell_atoms[ab + k];
        if (j == a) continue;
        const float4 pj = A.pos[j];
        if (r2_nofma(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z) > r2max) continue;
        const int d = j - a;
        bool keep = true;
        if (d >= -32 && d < 32) {
          if ((mask >> (d + 32)) & 1ull) keep = false;
        } else {
          for (int q = 0; q < far.y; ++q) {
            const int ent = A.far_list[far.x + q];
            if ((ent & 0x3fffffff) == j && (exclude_exc || !(ent & 0x40000000))) {
              keep = false;
              break;
            }
          }
        }
        if (keep) ok &= tile_insert(sh, (j - ab) >> 2, 1u << (i + 8 * ((j - ab) & 3)));
      }
    }
  }
  return __all_sync(0xffffffffu, ok);
}

// Test one candidate against every atom of the group and append the kept ones
// to the atoms' rows (ballot compaction keeps candidate order).  kCap: test
// each row against its capacity (the caller skips the tests for a chunk in
// which no row can reach it); kFull: the group has all eight atoms; kFar: some
// atom of the group has exclusions beyond the ±32 window.  An atom meets
// itself as a candidate at r^2 = 0 and is dropped by its own window bit
// (offset 0).
template <bool kCap, bool kFull, bool kFar>
__device__ __forceinline__ void group_test(const Arena& A, const GroupShared& sh, const float4 (&P)[8], int n_act,
                                           int a0, int g, bool valid, int j, float4 pj, float r2max,
                                           int exclude_exc, unsigned lt, int (&cnt)[8], unsigned& ovf) {
  int* const rows = A.nbr + (int64_t)g * kNbrCap * 8;  // tiled rows of the group's 8 atoms
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (!kFull && i >= n_act) break;
    const int ai = a0 + i;
    bool keep = valid && !(r2_nofma(pj.x - P[i].x, pj.y - P[i].y, pj.z - P[i].z) > r2max);
    if (keep) {
      const int d = j - ai;
      if (d >= -32 && d < 32) {
        if ((sh.mask[i] >> (d + 32)) & 1ull) keep = false;
      } else if (kFar) {
        const int2 far = sh.far[i];
        for (int q = 0; q < far.y; ++q) {
          const int ent = A.far_list[far.x + q];
          if ((ent & 0x3fffffff) == j && (exclude_exc || !(ent & 0x40000000))) {
            keep = false;
            break;
          }
        }
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int add = __popc(bal);
    if (kCap && cnt[i] + add > kNbrCap) {
      ovf |= 1u << i;
    } else {
      if (keep) {
        const int k = cnt[i] + __popc(bal & lt);  // same slot as nbr_index(ai, k)
        rows[(k >> 4) * 128 + (((i << 2) + (k & 3)) << 2) + ((k >> 2) & 3)] = j;
      }
      cnt[i] += add;
    }
  }
}

// Tile form of group_test: the candidate's pair bits with every atom of the
// group (same r^2 and exclusion tests) go into the group's tile table.
__device__ __forceinline__ bool group_test_tiles(const Arena& A, GroupShared& sh, const float4 (&P)[8], int n_act,
                                                 int a0, int ab, bool valid, int j, float4 pj, float r2max,
                                                 int exclude_exc) {
  unsigned m8 = 0u;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (i >= n_act) break;
    const int ai = a0 + i;
    bool keep = valid && j != ai;
    if (keep) keep = !(r2_nofma(pj.x - P[i].x, pj.y - P[i].y, pj.z - P[i].z) > r2max);
    if (keep) {
      const int d = j - ai;
      if (d >= -32 && d < 32) {
        if ((sh.mask[i] >> (d + 32)) & 1ull) keep = false;
      } else {
        const int2 far = sh.far[i];
        for (int q = 0; q < far.y; ++q) {
          const int ent = A.far_list[far.x + q];
          if ((ent & 0x3fffffff) == j && (exclude_exc || !(ent & 0x40000000))) {
            keep = false;
            break;
          }
        }
      }
    }
    if (keep) m8 |= 1u << i;
  }
  bool ok = true;
  if (m8) ok = tile_insert(sh, (j - ab) >> 2, m8 << (8 * ((j - ab) & 3)));
  return ok;
}

// Complete-mode rows of one 8-atom group, built together: the warp lists the
// cell-row runs of the union of the group's stencils (the rows and x-runs
// within r_list of the group's bounding box), packs their candidates into
// one stream of full 32-lane iterations, and tests every candidate against
// each atom of the group.  Each atom's row comes out identical to a scan of
// its own stencil: the union visits a superset of that atom's rows and
// x-runs in the same (z, y, x, atom) order, and a candidate is kept by the
// same r^2 and exclusion tests.
__device__ __forceinline__ void build_group(const Arena& A, int64_t g, int exclude_exc, int lane,
                                            GroupShared& sh) {
  const int a0 = (int)(g * 8);
  const int s = A.atom_sys[a0];
  SysDev* Sp = s >= 0 ? &A.sys[s] : nullptr;
  if (!Sp || !Sp->active || !Sp->rebuilding || Sp->status != 0) return;
  const int ab = Sp->atom_begin;
  const int n_act = min(8, ab + Sp->n_atoms - a0);
  const int dims[3] = {Sp->g_dims[0], Sp->g_dims[1], Sp->g_dims[2]};
  const float r2max = Sp->rlist2;
  const int* start = A.cell_start + Sp->cell_begin;
  // FP32 complete-mode lists are cluster-pair tiles (the production build
  // excludes the exception pairs, the parity build of prismq_build_neighbors
  // keeps them, as for rows)
  const bool tiles = uses_tiles(A, *Sp);
  float4 P[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) P[i] = A.pos[a0 + min(i, n_act - 1)];
  if (lane < n_act) {
    sh.mask[lane] = exclude_exc ? A.mask_all[a0 + lane] : A.mask_ref[a0 + lane];
    sh.far[lane] = A.far[a0 + lane];
  }
  // some atom of the group has exclusions beyond its ±32 window
  const bool far_any = __any_sync(0xffffffffu, lane < n_act && A.far[a0 + min(lane, n_act - 1)].y > 0);
  if (tiles) {
    for (int k = lane; k < kTileHash; k += 32) {
      sh.tkey[k] = 0;
      sh.tmask[k] = 0u;
    }
    if (lane == 0) sh.tcount = 0;
  }
  __syncwarp();
  float bl[3] = {P[0].x, P[0].y, P[0].z}, bh[3] = {P[0].x, P[0].y, P[0].z};
#pragma unroll
  for (int i = 1; i < 8; ++i) {
    bl[0] = fminf(bl[0], P[i].x);
    bl[1] = fminf(bl[1], P[i].y);
    bl[2] = fminf(bl[2], P[i].z);
    bh[0] = fmaxf(bh[0], P[i].x);
    bh[1] = fmaxf(bh[1], P[i].y);
    bh[2] = fmaxf(bh[2], P[i].z);
  }
  const float lox = Sp->g_lo[0], loy = Sp->g_lo[1], loz = Sp->g_lo[2];
  const float ivx = Sp->g_inv_edge[0], ivy = Sp->g_inv_edge[1], ivz = Sp->g_inv_edge[2];
  const float ey = 1.0f / ivy, ez = 1.0f / ivz;
  const float rl = sqrtf(r2max) + 1.0e-3f;
  const int z0 = max((int)((bl[2] - rl - loz) * ivz), 0), z1 = min((int)((bh[2] + rl - loz) * ivz), dims[2] - 1);
  const int y0 = max((int)((bl[1] - rl - loy) * ivy), 0), y1 = min((int)((bh[1] + rl - loy) * ivy), dims[1] - 1);
  const int ny = y1 - y0 + 1;
  const int n_rows = (z1 - z0 + 1) * ny;
  if (n_rows > kMaxRuns) {
    // a group that spans two distant chains: build its list atom by atom
    if (tiles) {
      bool ok = true;
      for (int i = 0; i < n_act; ++i) ok &= tile_atom(A, Sp, sh, a0 + i, i, lane, exclude_exc);
      const int nt = ok ? tile_flush(A, sh, g, ab, lane) : -1;
      if (nt < 0) {
        if (lane == 0) atomicOr(&Sp->status, kStNbrOverflow);
        return;
      }
      if (lane < n_act) A.xref[a0 + lane] = P[lane];
      __syncwarp();
      return;
    }
    for (int i = 0; i < n_act; ++i) {
      int count = -1;
      build_row(A, a0 + i, exclude_exc, lane, &count);
    }
    return;
  }
  // ---- the runs of candidates, one per (z, y) cell row, in scan order ----
  int total = 0;
  for (int r0 = 0; r0 < n_rows; r0 += 32) {
    const int r = r0 + lane;
    int b = 0, len = 0;
    if (r < n_rows) {
      const int z = z0 + r / ny, y = y0 + r % ny;
      const float sz = fmaxf(0.0f, fmaxf((loz + (float)z * ez) - bh[2], bl[2] - (loz + (float)(z + 1) * ez)));
      const float sy = fmaxf(0.0f, fmaxf((loy + (float)y * ey) - bh[1], bl[1] - (loy + (float)(y + 1) * ey)));
      const float mz = fmaxf(sz - 1.0e-3f, 0.0f), my = fmaxf(sy - 1.0e-3f, 0.0f);
      const float d2 = my * my + mz * mz;
      if (!(d2 > r2max)) {
        const float xr = sqrtf(r2max - d2) + 1.0e-3f;
        const int x0 = max((int)((bl[0] - xr - lox) * ivx), 0);
        const int x1 = min((int)((bh[0] + xr - lox) * ivx), dims[0] - 1);
        if (x0 <= x1) {
          const int rowc = y * dims[0] + z * dims[0] * dims[1];
          b = start[rowc + x0];
          len = start[rowc + x1 + 1] - b;
        }
      }
    }
    int incl = len;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (r < n_rows) {
      sh.run_b[r] = b;
      sh.run_off[r] = total + incl - len;
    }
    total += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) sh.run_off[n_rows] = total;
  __syncwarp();
  // ---- the packed candidate stream, software-pipelined: while chunk c is
  // tested, the position of chunk c+1 and the atom index of chunk c+2 are
  // in flight.  Each lane walks the runs forward (candidate c is in run r
  // when run_off[r] <= c < run_off[r+1]; chunks advance by 32, so the walk
  // moves a step or two per chunk). ----
  int run = 0;
  auto locate = [&](int cc) -> int {  // sorted-atom index of candidate cc (cc < total), cc non-decreasing
    while (sh.run_off[run + 1] <= cc) ++run;
    return sh.run_b[run] + (cc - sh.run_off[run]);
  };
  int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned ovf = 0u;
  const unsigned lt = (1u << lane) - 1u;
  int c = lane;
  int j = c < total ? A.cell_atoms[ab + locate(c)] : -1;
  int j1 = c + 32 < total ? A.cell_atoms[ab + locate(c + 32)] : -1;
  float4 pj = j >= 0 ? A.pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  bool tok = true;
  for (int c0 = 0; c0 < total; c0 += 32) {
    const bool valid = c < total;
    const float4 p1 = j1 >= 0 ? A.pos[j1] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int j2 = c + 64 < total ? A.cell_atoms[ab + locate(c + 64)] : -1;
    if (tiles) {
      tok &= group_test_tiles(A, sh, P, n_act, a0, ab, valid, j, pj, r2max, exclude_exc);
    } else {
      // a chunk adds at most 32 entries to a row
      int most = cnt[0];
#pragma unroll
      for (int i = 1; i < 8; ++i) most = max(most, cnt[i]);
      if (most <= kNbrCap - 32 && n_act == 8 && !far_any)
        group_test<false, true, false>(A, sh, P, n_act, a0, (int)g, valid, j, pj, r2max, exclude_exc, lt, cnt, ovf);
      else
        group_test<true, false, true>(A, sh, P, n_act, a0, (int)g, valid, j, pj, r2max, exclude_exc, lt, cnt, ovf);
    }
    c += 32;
    j = j1;
    pj = p1;
    j1 = j2;
  }
  if (tiles) {
    const int nt = __all_sync(0xffffffffu, tok) ? tile_flush(A, sh, g, ab, lane) : -1;
    if (nt < 0) {
      if (lane == 0) atomicOr(&Sp->status, kStNbrOverflow);
      return;
    }
    if (lane < n_act) A.xref[a0 + lane] = P[lane];
    __syncwarp();
    return;
  }
  if (ovf) {
    if (lane == 0) atomicOr(&Sp->status, kStNbrOverflow);
    return;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (lane == i && i < n_act) {
      A.nnbr[a0 + i] = cnt[i];
      A.xref[a0 + i] = P[i];
    }
  __syncwarp();
}

// Warps walk the queued 8-atom groups round-robin (`dynamic` 0), or take
// them one at a time from a shared counter (work_ctl[2], `dynamic` 1), so
// that a warp that drew cheap groups takes more of them; which warp builds a
// group does not change its rows.  The force kernel that follows in the same
// stream clears the queue and the counter.  Complete lists are built a group
// at a time; REF27 lists (parity only) atom by atom with the reference's own
// 27-cell stencil.
__global__ void __launch_bounds__(kNbrThreads, 3) k_nbr_build(Arena A, int64_t n_span, int exclude_exc,
                                                              int dynamic) {
  extern __shared__ __align__(16) unsigned char nbr_smem[];
  GroupShared* sh = reinterpret_cast<GroupShared*>(nbr_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    // a launch for the tile layout carries each warp's table after the records
    unsigned char* tab = nbr_smem + sizeof(GroupShared) * (kNbrThreads / 32) + warp * kTileTableBytes;
    sh[warp].tkey = A.pair_layout == 1 ? reinterpret_cast<int*>(tab) : nullptr;
    sh[warp].tmask = A.pair_layout == 1 ? reinterpret_cast<unsigned*>(tab + kTileHash * sizeof(int)) : nullptr;
  }
  __syncwarp();
  const int64_t gw = (int64_t)blockIdx.x * (kNbrThreads / 32) + warp;
  const int64_t n_warps = (int64_t)gridDim.x * (kNbrThreads / 32);
  const int64_t n_groups = A.work_ctl[0];
  // the queue length, kept for the force launch that follows (which clears
  // work_ctl[0] as it starts)
  if (blockIdx.x == 0 && threadIdx.x == 0) A.work_ctl[3] = (int)n_groups;
  if (gw >= n_groups) return;  // warps beyond the queue length leave at once
  for (int64_t v = gw;;) {
    if (dynamic) {
      int t = 0;
      if (lane == 0) t = atomicAdd(&A.work_ctl[2], 1);
      v = __shfl_sync(0xffffffffu, t, 0);
    }
    if (v >= n_groups) break;
    const int64_t g = A.work[v];
    if (!dynamic) v += n_warps;
    if (g * 8 >= n_span) continue;
    const int s = A.atom_sys[g * 8];
    if (s >= 0 && A.sys[s].nbr_mode == 1) {
      for (int i = 0; i < 8; ++i) {
        int count = -1;
        if (g * 8 + i < n_span) build_row(A, (int)(g * 8 + i), exclude_exc, lane, &count);
      }
    } else {
      build_group(A, g, exclude_exc, lane, sh[warp]);
    }
  }
}

// ---- the cell sort of large systems, grid-wide (a system of 100,000 atoms
// has ~50,000 cells: one CTA would walk them in sequence).  The same cell
// assignment, prefix sum and per-cell order as the single-CTA path, so the
// rows that follow are identical. ----
constexpr int kBigThreads = 256;

__global__ void __launch_bounds__(kBigThreads) k_big_count(Arena A) {
  const int nb = A.work_ctl[1];
  for (int k = 0; k < nb; ++k) {
    const SysDev* Sp = &A.sys[A.big_list[k]];
    float lo[3], iv[3];
    int dims[3];
    grid_of(Sp, lo, iv, dims);
    int* start = A.cell_start + Sp->cell_begin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Sp->n_atoms; i += gridDim.x * blockDim.x) {
      const int a = Sp->atom_begin + i;
      const int c = cell_of(A.pos[a], Sp->nbr_mode, lo, iv, dims);
      A.atom_cell[a] = c;
      atomicAdd(&start[c + 1], 1);
    }
  }
}

// One block per large system: the exclusive prefix over its cells in tiles
// of 1024 cells (one per thread, coalesced), each tile a block-wide scan
// plus the running total of the tiles before it; the next tile's counts load
// while the current one is scanned.
__global__ void __launch_bounds__(1024) k_big_scan(Arena A) {
  __shared__ int wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = A.work_ctl[1];
  for (int k = blockIdx.x; k < nb; k += gridDim.x) {
    SysDev* Sp = &A.sys[A.big_list[k]];
    const int nc = Sp->nbr_mode == 1 ? Sp->ref_dims[0] * Sp->ref_dims[1] * Sp->ref_dims[2]
                                     : Sp->g_dims[0] * Sp->g_dims[1] * Sp->g_dims[2];
    int* start = A.cell_start + Sp->cell_begin;
    int* cursor = start + (Sp->cell_cap + 1);
    bool ovf = false;
    int carry = 0;
    int v_next = tid < nc ? start[tid + 1] : 0;
    for (int base = 0; base < nc; base += 1024) {
      const int c = base + tid;
      const int v = v_next;
      v_next = c + 1024 < nc ? start[c + 1024 + 1] : 0;
      ovf |= v > kCellSortCap;
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) wsum[warp] = x;
      __syncthreads();
      if (warp == 0) {
        int w = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += y;
        }
        wsum[lane] = w;
      }
      __syncthreads();
      const int incl = carry + x + (warp > 0 ? wsum[warp - 1] : 0);
      if (c < nc) {
        cursor[c] = incl - v;
        start[c + 1] = incl;
      }
      carry += wsum[31];
      __syncthreads();  // wsum is rewritten by the next tile
    }
    if (__syncthreads_or(ovf) && tid == 0) atomicOr(&Sp->status, kStCellOverflow);
  }
}

__global__ void __launch_bounds__(kBigThreads) k_big_scatter(Arena A) {
  const int nb = A.work_ctl[1];
  for (int k = 0; k < nb; ++k) {
    const SysDev* Sp = &A.sys[A.big_list[k]];
    if (Sp->status != 0) continue;
    int* cursor = A.cell_start + Sp->cell_begin + (Sp->cell_cap + 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Sp->n_atoms; i += gridDim.x * blockDim.x) {
      const int a = Sp->atom_begin + i;
      const int slot = atomicAdd(&cursor[A.atom_cell[a]], 1);
      A.cell_atoms[Sp->atom_begin + slot] = a;
    }
  }
}

__global__ void __launch_bounds__(kBigThreads) k_big_sort(Arena A) {
  extern __shared__ int sm[];  // per-warp scratch: 8 * kCellSortCap ints
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = A.work_ctl[1];
  int* buf = sm + warp * kCellSortCap;
  for (int k = 0; k < nb; ++k) {
    const SysDev* Sp = &A.sys[A.big_list[k]];
    if (Sp->status != 0) continue;
    const int nc = Sp->nbr_mode == 1 ? Sp->ref_dims[0] * Sp->ref_dims[1] * Sp->ref_dims[2]
                                     : Sp->g_dims[0] * Sp->g_dims[1] * Sp->g_dims[2];
    const int* start = A.cell_start + Sp->cell_begin;
    for (int c = blockIdx.x * (kBigThreads / 32) + warp; c < nc; c += gridDim.x * (kBigThreads / 32)) {
      const int b = start[c];
      sort_cell(A.cell_atoms + Sp->atom_begin + b, start[c + 1] - b, buf, lane);
    }
  }
}

void launch_big_cells(const Arena& A, int64_t max_big_atoms, cudaStream_t st) {
  if (max_big_atoms <= 0) return;
  static bool attr = false;
  const size_t smem = (size_t)(kBigThreads / 32) * kCellSortCap * sizeof(int);
  if (!attr) {
    cudaFuncSetAttribute(k_big_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  // The kernels stride over atoms and cells, and they sit in every step's
  // graph while a large system is resident, so their grids stay at a few
  // blocks per SM: on steps without a rebuild every block only reads the
  // empty work list and leaves.
  static int cap_blocks = 0;
  if (!cap_blocks) {
    int dev = 0, n_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    cap_blocks = 4 * std::max(n_sm, 1);
  }
  const unsigned atoms_blocks =
      (unsigned)std::min<int64_t>((max_big_atoms + kBigThreads - 1) / kBigThreads, cap_blocks);
  const unsigned cell_blocks = (unsigned)std::min<int64_t>((max_big_atoms / 2 + 8) / 8, cap_blocks);  // cells <= atoms / 2
  k_big_count<<<atoms_blocks, kBigThreads, 0, st>>>(A);
  k_big_scan<<<1, 1024, 0, st>>>(A);
  k_big_scatter<<<atoms_blocks, kBigThreads, 0, st>>>(A);
  k_big_sort<<<cell_blocks, kBigThreads, smem, st>>>(A);
}

void launch_control_cells(const Arena& A, int n_sys, int mode, int nbr_override, cudaStream_t st) {
  if (n_sys <= 0) return;
  const size_t smem = (size_t)(kCtlThreads / 32) * kCellSortCap * sizeof(int);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_control_cells, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_control_cells<<<n_sys, kCtlThreads, smem, st>>>(A, mode, nbr_override);
}

// Grid: the CTAs that fit on the GPU at once (fewer for a short span).  With
// `round_robin` (a builder beside the overlapped force launch of a
// many-system step) the warps stride over the queue round-robin; otherwise
// (priming, or a step of one or two systems, where a rebuild has nothing to
// overlap) they take groups from the shared counter, which on the
// 100,000-atom system took the builder from 0.184 to 0.172 ms per step
// against one warp per group.  The counter is no help beside the force
// launch: the builder then finishes sooner but takes more of the GPU from it
// (256 systems: 0.877 against 0.868 ms per step).
void launch_nbr_build(const Arena& A, int64_t n_atoms_span, int exclude_exceptions, cudaStream_t st,
                      bool round_robin) {
  if (n_atoms_span <= 0) return;
  // the per-warp tile tables only in launches for the tile layout: a row
  // build leaves that shared memory to L1
  const size_t smem_rows = sizeof(GroupShared) * (kNbrThreads / 32);
  const size_t smem_max = smem_rows + kTileTableBytes * (kNbrThreads / 32);
  const size_t smem = A.pair_layout == 1 ? smem_max : smem_rows;
  static int resident = 0;  // CTAs that fit on the GPU at once
  if (!resident) {
    int dev = 0, n_sm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_nbr_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_nbr_build, kNbrThreads, smem_max);
    resident = std::max(1, n_sm) * std::max(1, per_sm);
  }
  const int64_t groups = (n_atoms_span + 7) / 8;
  const int64_t per_group = (groups + kNbrThreads / 32 - 1) / (kNbrThreads / 32);
  const int grid = (int)std::min<int64_t>(per_group, resident);
  k_nbr_build<<<grid, kNbrThreads, smem, st>>>(A, n_atoms_span, exclude_exceptions, round_robin ? 0 : 1);
}

}  // namespace pq
