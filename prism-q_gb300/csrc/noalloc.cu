// Neighbour rows without any device allocation.
//
// Some callers of this library cannot call cudaMalloc while they run: a
// serving process that reserves its whole HBM budget for job arenas up front,
// or a host loop whose allocator policy forbids device allocations after
// start-up because cudaMalloc/cudaFree synchronise the device and fragment
// memory.  For them this file offers one entry point,
// prismq_neighbor_rows_noalloc(), which builds the complete neighbour rows of
// a point set (every pair within the list radius, as the batched builder's
// complete mode does) into buffers the caller already owns.
//
// The cell lists the builder needs live in one file-scope __device__ array of
// fixed size (kNaScratchInts ints, about 0.8 MB), which every GPU that loads
// the library holds until the process exits.  Host code may not pass that
// array's name to a kernel — on the host it is only a stand-in for the device
// symbol — so the first call on each device looks up its device address with
// cudaGetSymbolAddress while that device is current, and later calls reuse
// it.  That first call therefore does set-up work and should come before any
// stream capture.  The cached address belongs to the device's current
// context: after cudaDeviceReset (or any teardown of the primary context) the
// module is loaded again and the cache is stale, so this entry point must not
// be used across a device reset.  All calls share the one array: the kernels
// clear what must start at zero on every call, and calls that overlap on the
// GPU (two streams, two host threads) race on it and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/prismq_md.h"

namespace {

constexpr int kNaMaxAtoms = 65536;
constexpr int kNaMaxCells = 32768;
constexpr int kNaCellCap = 512;   // atoms per cell (sort scratch); more is reported as overflow
constexpr int kNaRowCapMax = 1024;
constexpr int kNaHeader = 16;     // [0] error bits, [1..3] dims, [4..6] lo (float bits), [7..9] inv edge
constexpr int kNaScratchInts = kNaHeader + 2 * (kNaMaxCells + 1) + 2 * kNaMaxAtoms;

static __device__ __align__(256) int g_na_scratch[kNaScratchInts];

constexpr int kNaErrCell = 1, kNaErrRow = 2;

std::mutex g_na_mu;
int* g_na_addr[64] = {nullptr};  // device address of g_na_scratch, per device ordinal

__device__ __forceinline__ float na_r2(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// One CTA: bounding box, grid of cells at least r/2 wide, counting sort and an
// ascending sort of each cell's atoms.
__global__ void __launch_bounds__(1024) k_na_cells(int* scr, const float* xyz, int n, float r) {
  extern __shared__ int sm[];
  __shared__ float red[6][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int* hdr = scr;
  int* start = scr + kNaHeader;
  int* cursor = start + (kNaMaxCells + 1);
  int* acell = cursor + (kNaMaxCells + 1);
  int* catoms = acell + kNaMaxAtoms;
  float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = tid; i < n; i += 1024)
    for (int d = 0; d < 3; ++d) {
      mn[d] = fminf(mn[d], xyz[3 * i + d]);
      mx[d] = fmaxf(mx[d], xyz[3 * i + d]);
    }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; ++d) {
      mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      red[d][warp] = mn[d];
      red[3 + d][warp] = mx[d];
    }
  __syncthreads();
  if (tid == 0) {
    hdr[0] = 0;
    int nd[3];
    float ext[3], lo[3];
    for (int d = 0; d < 3; ++d) {
      float a = red[d][0], b = red[3 + d][0];
      for (int w = 1; w < 32; ++w) {
        a = fminf(a, red[d][w]);
        b = fmaxf(b, red[3 + d][w]);
      }
      lo[d] = a;
      ext[d] = fmaxf(b - a, 1.0e-3f);
      // Cells at least 0.5005 r wide, so the ±2 stencil reaches 1.001 r: the
      // 1e-3 margin covers the float rounding of (x - lo) * inv, about
      // nd * 1.2e-7 cells per atom.  Capping nd (here, or in the product
      // loop below) only widens the cells.
      const float q = ext[d] / (r * 0.5005f);
      nd[d] = q >= 1.0f ? (int)fminf(q, 1024.0f) : 1;
    }
    while ((long long)nd[0] * nd[1] * nd[2] > kNaMaxCells) {
      int big = 0;
      if (nd[1] > nd[big]) big = 1;
      if (nd[2] > nd[big]) big = 2;
      nd[big] -= 1;
    }
    for (int d = 0; d < 3; ++d) {
      hdr[1 + d] = nd[d];
      hdr[4 + d] = __float_as_int(lo[d]);
      hdr[7 + d] = __float_as_int((float)nd[d] / ext[d]);
    }
  }
  __syncthreads();
  const int dx = hdr[1], dy = hdr[2], dz = hdr[3];
  const float lx = __int_as_float(hdr[4]), ly = __int_as_float(hdr[5]), lz = __int_as_float(hdr[6]);
  const float ix = __int_as_float(hdr[7]), iy = __int_as_float(hdr[8]), iz = __int_as_float(hdr[9]);
  const int ncell = dx * dy * dz;
  for (int c = tid; c <= ncell; c += 1024) start[c] = 0;
  __syncthreads();
  for (int i = tid; i < n; i += 1024) {
    int cx = (int)((xyz[3 * i] - lx) * ix), cy = (int)((xyz[3 * i + 1] - ly) * iy),
        cz = (int)((xyz[3 * i + 2] - lz) * iz);
    cx = min(max(cx, 0), dx - 1);
    cy = min(max(cy, 0), dy - 1);
    cz = min(max(cz, 0), dz - 1);
    const int c = cx + cy * dx + cz * dx * dy;
    acell[i] = c;
    atomicAdd(&start[c + 1], 1);
  }
  __syncthreads();
  // exclusive prefix of the cell counts, 1024 cells per pass (warp scans plus
  // a carry), run on every call
  {
    __shared__ int wsum[32];
    __shared__ int carry;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ncell; base += 1024) {
      const int c = base + tid;
      const int v = c < ncell ? start[c + 1] : 0;
      if (v > kNaCellCap) atomicOr(&hdr[0], kNaErrCell);
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
      if (tid == 1023) carry = incl;
      __syncthreads();
    }
  }
  if (hdr[0]) return;
  for (int i = tid; i < n; i += 1024) catoms[atomicAdd(&cursor[acell[i]], 1)] = i;
  __syncthreads();
  int* buf = sm + warp * kNaCellCap;
  for (int c = warp; c < ncell; c += 32) {
    const int b = start[c], e = start[c + 1], m = e - b;
    if (m <= 1) continue;
    int p2 = 1;
    while (p2 < m) p2 <<= 1;
    for (int k = lane; k < p2; k += 32) buf[k] = k < m ? catoms[b + k] : 0x7fffffff;
    __syncwarp();
    for (int w = 2; w <= p2; w <<= 1)
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
    for (int k = lane; k < m; k += 32) catoms[b + k] = buf[k];
    __syncwarp();
  }
}

// Warp per atom: scan the ±2 cell stencil row by row (each row of five cells is
// one contiguous run of sorted atoms), keep !(r2 > r^2), write row-major.
__global__ void __launch_bounds__(256) k_na_rows(int* scr, const float* xyz, int n, float r2max, int row_cap,
                                                 int* rows, int* counts) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= n) return;
  int* hdr = scr;
  const int* start = scr + kNaHeader;
  const int* acell = start + 2 * (kNaMaxCells + 1);
  const int* catoms = acell + kNaMaxAtoms;
  if (hdr[0] & kNaErrCell) {
    if (lane == 0) counts[i] = -1;
    return;
  }
  const int dx = hdr[1], dy = hdr[2], dz = hdr[3];
  const int c = acell[i];
  const int cx = c % dx, cy = (c / dx) % dy, cz = c / (dx * dy);
  const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
  int* row = rows + (size_t)i * row_cap;
  int cnt = 0;
  bool over = false;
  for (int oz = -2; oz <= 2; ++oz) {
    const int z = cz + oz;
    if (z < 0 || z >= dz) continue;
    for (int oy = -2; oy <= 2; ++oy) {
      const int y = cy + oy;
      if (y < 0 || y >= dy) continue;
      const int x0 = max(cx - 2, 0), x1 = min(cx + 2, dx - 1);
      const int base = y * dx + z * dx * dy;
      const int b = start[base + x0], e = start[base + x1 + 1];
      for (int k0 = b; k0 < e; k0 += 32) {
        const int k = k0 + lane;
        int j = 0;
        bool keep = false;
        if (k < e) {
          j = catoms[k];
          if (j != i) {
            const float r2 = na_r2(xyz[3 * j] - px, xyz[3 * j + 1] - py, xyz[3 * j + 2] - pz);
            keep = !(r2 > r2max);
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        const int add = __popc(bal);
        if (cnt + add > row_cap) {
          over = true;
        } else {
          if (keep) row[cnt + __popc(bal & ((1u << lane) - 1u))] = j;
          cnt += add;
        }
      }
    }
  }
  if (lane == 0) {
    counts[i] = over ? -1 : cnt;
    if (over) atomicOr(&hdr[0], kNaErrRow);
  }
}

}  // namespace

namespace pq {
void set_last_error(const std::string& msg);  // engine.cu: the message prismq_last_error() returns
}

static prismq_status na_fail(prismq_status st, const std::string& msg) {
  pq::set_last_error(msg);
  return st;
}

extern "C" prismq_status prismq_neighbor_rows_noalloc(const float* d_xyz, int32_t n_atoms, float list_radius,
                                                      int32_t row_cap, int32_t* d_rows, int32_t* d_counts,
                                                      void* stream) {
  if (n_atoms < 1 || n_atoms > kNaMaxAtoms) {
    return na_fail(PRISMQ_E_CAPACITY, "prismq_neighbor_rows_noalloc: n_atoms must be 1.." + std::to_string(kNaMaxAtoms));
  }
  if (row_cap < 1 || row_cap > kNaRowCapMax) {
    return na_fail(PRISMQ_E_CAPACITY, "prismq_neighbor_rows_noalloc: row_cap must be 1.." + std::to_string(kNaRowCapMax));
  }
  if (!(list_radius > 0.0f) || !d_xyz || !d_rows || !d_counts) {
    return na_fail(PRISMQ_E_INVALID, "prismq_neighbor_rows_noalloc: invalid argument");
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    return na_fail(PRISMQ_E_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  int* scr = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
      // first call on this device (current here): resolve the symbol's device address
      e = cudaGetSymbolAddress((void**)&g_na_addr[dev], g_na_scratch);
      if (e != cudaSuccess) {
        g_na_addr[dev] = nullptr;
        return na_fail(PRISMQ_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      const int smem = 32 * kNaCellCap * (int)sizeof(int);
      e = cudaFuncSetAttribute(k_na_cells, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) {
        g_na_addr[dev] = nullptr;
        return na_fail(PRISMQ_E_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
      }
    }
    scr = g_na_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_na_cells<<<1, 1024, 32 * kNaCellCap * sizeof(int), st>>>(scr, d_xyz, n_atoms, list_radius);
  const float r2 = list_radius * list_radius;
  k_na_rows<<<(n_atoms + 7) / 8, 256, 0, st>>>(scr, d_xyz, n_atoms, r2, row_cap, d_rows, d_counts);
  int err = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, scr, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    return na_fail(PRISMQ_E_CUDA, std::string("prismq_neighbor_rows_noalloc: ") + cudaGetErrorString(e));
  }
  if (err & kNaErrCell) {
    return na_fail(PRISMQ_E_CELL_OVERFLOW, "prismq_neighbor_rows_noalloc: a cell held more than 512 atoms");
  }
  if (err & kNaErrRow) {
    return na_fail(PRISMQ_E_NEIGHBOR_OVERFLOW, "prismq_neighbor_rows_noalloc: a row exceeded row_cap (its count is -1)");
  }
  return PRISMQ_OK;
}
