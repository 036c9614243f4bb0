// Device data layout of the batched MD arena and the launchers of each kernel.
//
// All resident systems share one global atom index space.  Per-atom streams
// are SoA float4 (position+charge, velocity+mass), float2 LJ, int64 forces
// (three planes); bonded terms, exceptions and constraint units refer to
// global atom indices.  One SysDev record per system carries its parameters
// and the device-resident control state that a captured CUDA graph reads.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pq_protocol.h"

namespace pq {

constexpr int kNbrCap = 1024;     // neighbour row capacity per atom
constexpr int kLanes = 4;         // threads per atom in the force kernel (fixed: results depend on it)

// Row storage is tiled for the force kernel's warp shape (8 atoms x 4 lanes;
// lane q of atom a takes entries k = 4t + q).  Each lane's entries t..t+3
// (t a multiple of 4) are one aligned int4, and the 32 lanes' int4s of an
// 8-atom group are one contiguous 512-byte block:
//   group a/8, block t/4, lane slot (a%8)*4 + q, word t%4.
__host__ __device__ __forceinline__ int64_t nbr_index(int64_t a, int k) {
  const int t = k >> 2;
  return (a >> 3) * (kNbrCap * 8) + (t >> 2) * 128 + ((((int)(a & 7) << 2) + (k & 3)) << 2) + (t & 3);
}
// Cluster-pair tiles (FP32 complete-mode lists): an i-cluster is an aligned
// group of 8 consecutive atoms, a j-cluster an aligned group of 4; one tile
// {j-cluster, 32-bit mask} says which of the 8 x 4 pairs are in the list
// (bit i + 8 jj for atoms 8g + i and 4jc + jj).  Tiles of an i-cluster are
// stored in ascending j-cluster order, at most kTileCap of them.
constexpr int kTileCap = 768;
constexpr int kTileHash = 1024;  // per-warp build table (open addressing over j-clusters)
constexpr int kRefCellCap = 512;  // REF27 cell capacity (MAX_ATOMS_PER_CELL)
constexpr int kRefMaxDim = 32;    // REF27 cells per axis (MAX_CELLS_PER_DIM)

// status bits of SysDev::status
constexpr int kStShake = 1;
constexpr int kStRattle = 2;
constexpr int kStCellOverflow = 4;
constexpr int kStNbrOverflow = 8;
constexpr int kStNonfinite = 16;

// Bonded terms carry, per member, the term's position in that member's
// incidence list of its kind (`pos`), so a term evaluated once can drop each
// member's contribution into the slot that member's gather reads.
struct BondT {
  int i, j;
  float r0, k;
  int pos;  // pos_i | pos_j << 16
};
struct AngleT {
  int i, j, k;
  float theta0, kf;
  int pos;  // pos_i | pos_j << 10 | pos_k << 20
};
constexpr int kMaxPeriodicity = 64;  // torsion periodicities accepted by the lowering
struct DihT {
  int i, j, k, l;
  int n;
  float phase, kf;
  float cos_ph, sin_ph;  // cos and sin of the phase, from the host in double
  int pos;  // 8 bits per member
};
// One exact 1-4 exception pair (each pair once), with its rank in each
// member's ascending exception list.
struct ExcT {
  int i, j;
  float qq, sig, eps;
  int pos;  // pos_i | pos_j << 16
};

// Kinds of the per-group term references (ref = kind << 29 | term index).
constexpr int kRefBond = 0, kRefAngle = 1, kRefDih = 2, kRefExc = 3;
constexpr int kForceGroup = 32;  // atoms per force block (128 threads, 4 lanes per atom)
constexpr int kMaxGroupSlots = 2048;  // bonded + exception incidences of one group (shared-memory slots)

// A constraint unit: one H cluster (central + up to 3 H) or one lone atom.
struct Unit {
  int a[4];  // a[0] central / lone atom, a[1..3] hydrogens or -1
  int nh;    // hydrogens (0 for a lone atom), -1 for an inactive slot
  int sys;
  float r0[3];
  float inv_mc, inv_mh;
  int pad;
};

struct SysDev {
  // layout
  int atom_begin, n_atoms, unit_begin, n_units;
  int cell_begin, cell_cap;
  int active;
  int nbr_mode;  // 0 complete (production), 1 REF27 (parity only)
  // parameters
  float dt, temperature, gamma, c1;
  float rlist2, half_skin2;
  float ref_r2;  // REF27 list radius^2 = f32(cutoff^2) * 1.44f (fused_engine.rs:16674)
  float cut2;    // potential cutoff^2
  int rebuild_interval, com_interval, max_iter;
  uint32_t seed, stream;
  // REF27 grid fixed at admission (fused_engine.rs:12285-12330)
  float ref_origin[3];
  int ref_dims[3];
  // dynamic control state
  long long step;
  int steps_since_rebuild;
  int displaced;
  int rebuilding;
  int status;
  int built;       // a list has been built at least once
  int need_prime;  // set by the host when forces must be recomputed before stepping
  // grid of the last build (complete mode)
  float g_lo[3];
  float g_inv_edge[3];
  int g_dims[3];
  int pad1;
  double vcom[3];
  long long n_rebuilds;  // list builds so far (statistics)
  // constraint convergence (reference: SHAKE 1e-4 on |r^2-L^2|/L^2, RATTLE 1e-5)
  float shake_tol, rattle_tol;
  int check64;  // 1: constraint residuals and multipliers evaluated in FP64
  int pad2;
  double c1d;   // exp(-γ·dt/2) in double (FP64 batches)
  // The fields above (dt, temperature, gamma, c1, c1d) are the parameters of
  // the step whose pre-force phases run next.  The post-force phases of a
  // step run in the next launch, so the control kernel carries that step's
  // values forward here before it moves the current set to the next step.
  float post_dt, post_temperature, post_gamma, post_c1;
  double post_c1d;
  ProtocolDev proto;  // proto.on: the control kernel evaluates T, γ, dt every step
  // Set by k_decide at the start of a step.  branch_a: the system's forces
  // wait for this step's control and row-building launches (it rebuilds its
  // list, or its COM removal and pre-force phases run in the control
  // kernel); the other systems' forces run concurrently with those launches.
  int branch_a;
  int com_pending;  // this step removes the COM velocity in the control kernel
};

// Per-atom incidence into bonded term arrays (reference: atom_bond_list etc.,
// fused_engine.rs:11704-11745).  Entries are term_index*4 + position.
struct Incidence {
  int b_beg, a_beg, d_beg;
  int counts;  // nb | na << 8 | nd << 16
};

struct Arena {
  int64_t atom_cap = 0, unit_cap = 0, bond_cap = 0, angle_cap = 0, dih_cap = 0, inc_cap = 0,
          ex_cap = 0, far_cap = 0, cell_cap = 0, exc_cap = 0, gref_cap = 0;
  int sys_cap = 0;
  // per atom
  float4* pos = nullptr;   // x y z q
  float4* vel = nullptr;   // vx vy vz mass
  float2* lj = nullptr;    // sigma/2, sqrt(eps)
  float4* xref = nullptr;  // positions at the last list build
  long long* f = nullptr;  // 3 planes of atom_cap
  double* pe = nullptr;    // 5 planes (bond, angle, dihedral, exception, nonbonded) of atom_cap
  int* atom_sys = nullptr;
  unsigned long long* mask_all = nullptr;  // exclusion window bits, offsets -32..31 (offset 0: the atom itself)
  unsigned long long* mask_ref = nullptr;  // same without exception pairs
  int2* far = nullptr;                     // {begin, count} into far_list
  int* far_list = nullptr;                 // partner | (is_exception << 30)
  Incidence* inc = nullptr;
  int* inc_list = nullptr;
  int2* ex_idx = nullptr;     // {begin, count}
  int* ex_partner = nullptr;  // global partner index
  float4* ex_par = nullptr;   // qq, sigma, epsilon, 0
  ExcT* exc = nullptr;        // exception pairs, each once
  // per 32-atom force group: {begin, count} into grp_refs, the terms with a
  // member in the group
  int2* grp = nullptr;
  int* grp_refs = nullptr;
  // terms
  BondT* bonds = nullptr;
  AngleT* angles = nullptr;
  DihT* dihs = nullptr;
  // constraint units, and the order the integrate grid walks them in: every
  // system's 3-hydrogen units, then 2, 1, 0, as ranges of units (range r
  // holds order_range[r].y units from order_range[r].x; order_prefix[r] is
  // the walk position of its first unit)
  Unit* units = nullptr;
  int2* order_range = nullptr;  // [4 * sys_cap]
  int* order_prefix = nullptr;  // [4 * sys_cap + 1]
  int n_ranges = 0;
  // OU normals drawn ahead of the integrate launch, per atom: [0, atom_cap)
  // for post(s-1), [atom_cap, 2 atom_cap) for pre(s)
  float4* noise = nullptr;
  // lists
  int* nbr = nullptr;   // tiled rows, see nbr_index()
  int* nnbr = nullptr;  // row lengths
  // cluster-pair tiles: pair_layout 1 selects them for FP32 complete-mode
  // systems (0, the default: rows for every system)
  int pair_layout = 0;
  int2* tiles = nullptr;  // [atom_cap / 8][kTileCap] {j-cluster, mask}
  int* ntile = nullptr;   // [atom_cap / 8] tiles per i-cluster
  int* cell_start = nullptr;  // per system: cell_cap+1 entries
  int* cell_atoms = nullptr;  // per atom (sorted by cell)
  int* atom_cell = nullptr;
  // work list of 8-atom groups to (re)build; work_ctl[0] = queued groups
  int* work = nullptr;
  int* work_ctl = nullptr;  // [0] queued groups, [1] systems in big_list
  int* big_list = nullptr;  // rebuilding systems of >= kBigSortAtoms atoms (the control kernel appends)
  // systems
  SysDev* sys = nullptr;
  // FP64 batches only (null otherwise): the state and forces of the
  // FP64-everywhere run; pos/vel above then hold its FP32 rounding, which the
  // cell and neighbour-row kernels read.
  int fp64 = 0;
  double4_32a* pos64 = nullptr;  // x y z q
  double4_32a* vel64 = nullptr;  // vx vy vz mass
  double* f64 = nullptr;     // 3 planes of atom_cap
  double2* lj64 = nullptr;   // sigma/2, sqrt(eps) in double
};

// Whether a system's list is cluster-pair tiles (else neighbour rows).
__host__ __device__ __forceinline__ bool uses_tiles(const Arena& A, const SysDev& S) {
  return A.pair_layout == 1 && !A.fp64 && S.nbr_mode == 0;
}

// K2 modes
constexpr int kCtlPrime = 0;  // force a rebuild, no COM, no step increment
constexpr int kCtlStep = 1;   // deferred COM pre-phase, rebuild decision, step increment
constexpr int kCtlForce = 2;  // force a rebuild inside a step sequence (after set_positions)

// K1 modes
constexpr int kIntPre = 1;
constexpr int kIntPost = 2;
constexpr int kIntBoth = 3;

// launchers (nbr.cu, force.cu, integrate.cu)
void launch_control_cells(const Arena& A, int n_sys, int mode, int nbr_mode_override,
                          cudaStream_t st);
// Systems of at least this many atoms have their cells sorted by grid-wide
// kernels (launch_big_cells) instead of inside their control block.
constexpr int kBigSortAtoms = 16384;
void launch_big_cells(const Arena& A, int64_t max_big_atoms, cudaStream_t st);
// The per-system schedule decision of a step (one thread per system).
void launch_decide(const Arena& A, int n_sys, cudaStream_t st);
// Force launch selections.
constexpr int kSelAll = 0, kSelRebuilding = 1, kSelBranchA = 2, kSelBranchB = 3;
void launch_nbr_build(const Arena& A, int64_t n_atoms_span, int exclude_exceptions,
                      cudaStream_t st, bool round_robin = false);
// group_slots: the largest number of bonded + exception incidences of one
// 32-atom group among the resident systems (sizes the shared-memory slots).
// sel: kSelAll, kSelRebuilding (systems rebuilt by the preceding control
// pass), kSelBranchA / kSelBranchB (the two halves of an overlapped step).
void launch_force(const Arena& A, int64_t n_atoms_span, bool energy, cudaStream_t st,
                  int sel = kSelAll, int variant = 0, int group_slots = 0);
int force_variant_count();
void force_variant_shape(int variant, int* block, int* min_blocks);
int force_variant_prefetch(int variant);  // row-index L2 prefetch distance (iterations; 0 = none)
// check64_pass: 0 = systems with FP32 constraint checks, 1 = systems with FP64
// checks (FP32 batches launch one pass per kind present); FP64 batches ignore it.
void launch_integrate(const Arena& A, int64_t n_units_span, int mode, cudaStream_t st, int check64_pass = 0);
// Draw the OU normals the next integrate launch of `mode` uses.
void launch_noise(const Arena& A, int64_t n_atoms_span, int mode, cudaStream_t st);
void launch_debug_phases(const Arena& A, int64_t n_units_span, int set, long long step,
                         cudaStream_t st);
constexpr int kEnergyOut = 15;  // per system: 5 potential planes, kinetic, 3x3 virial
void launch_energy_reduce(const Arena& A, int n_sys, double* out, cudaStream_t st);

}  // namespace pq
