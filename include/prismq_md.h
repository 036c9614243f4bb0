/*
 * prismq_md.h — C ABI of the GB300-native Prism-Q classical MD step.
 *
 * The library (libprismq_md.so) implements, as hand-written sm_103a CUDA
 * kernels, the hot path of Prism-Q's NhsAmberFusedEngine:
 *   cell-list neighbour build, AMBER ff14SB bonded forces, 10 Å potential-
 *   shifted vacuum Coulomb + Lennard-Jones, the BAOAB/OVRVO Langevin phases
 *   (OU, kick, drift) with SHAKE/RATTLE on X–H bonds under HMR.
 *
 * Conventions
 *   - Units are the reference engine's: Å, ps, amu, kcal/mol, e.
 *   - Positions, velocities and forces cross this boundary as host AoS
 *     float[3*N] (x0,y0,z0,x1,...), the layout of NhsAmberFusedEngine's
 *     get_positions/get_velocities (crates/prism-nhs/src/fused_engine.rs:24117,
 *     :20939).  Internally the library keeps SoA float4 streams and int64
 *     fixed-point forces at 2^-32 kcal/mol/Å.
 *   - Every call returns a prismq_status; PRISMQ_OK is 0.  Device-side
 *     failures (constraint non-convergence, list overflow, ...) never trap:
 *     they set a per-system status word that the next host call reports.
 *     prismq_last_error() returns the calling thread's last message.
 *   - The library owns all device memory.  Caller buffers are host memory.
 *   - A system or batch handle is externally synchronised (one thread at a
 *     time); a server handle is internally locked.
 *   - Pointers passed in a prismq_topology are read during the call only.
 */
#ifndef PRISMQ_MD_H
#define PRISMQ_MD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PRISMQ_ABI_VERSION 3

typedef enum prismq_status {
  PRISMQ_OK = 0,
  PRISMQ_E_INVALID = 1,          /* bad argument / topology (host validation) */
  PRISMQ_E_CUDA = 2,             /* CUDA runtime error */
  PRISMQ_E_NO_DEVICE = 3,        /* no CUDA device visible */
  PRISMQ_E_CAPACITY = 4,         /* caller buffer or arena too small */
  PRISMQ_E_CELL_OVERFLOW = 5,    /* a cell held more atoms than the grid allows */
  PRISMQ_E_NEIGHBOR_OVERFLOW = 6,/* an atom's row or a cluster's tile list was full */
  PRISMQ_E_SHAKE = 7,            /* SHAKE did not converge in max_iter */
  PRISMQ_E_RATTLE = 8,           /* RATTLE did not converge in max_iter */
  PRISMQ_E_NONFINITE = 9,        /* NaN/Inf in state or forces */
  PRISMQ_E_BUSY = 10,            /* server queue full */
  PRISMQ_E_NOT_FOUND = 11
} prismq_status;

/* ---- topology (mirrors PrismPrepTopology, crates/prism-nhs/src/input.rs:1027-1140) ---- */

typedef struct prismq_bond {      /* input.rs:230 BondParam; U = k (r - r0)^2 (k pre-halved) */
  int32_t i, j;
  float r0, k;
} prismq_bond;

typedef struct prismq_angle {     /* input.rs:243 AngleParam; U = k (θ - θ0)^2, θ in radians */
  int32_t i, j, k;
  float theta0, force_k;
} prismq_angle;

typedef struct prismq_dihedral {  /* input.rs:541 DihedralParam; U = k (1 + cos(nφ - γ)), 1 <= n <= 64 */
  int32_t i, j, k, l;
  int32_t periodicity;
  float phase, force_k;
} prismq_dihedral;

typedef struct prismq_exception { /* input.rs:581 NonbondedExceptionParam (exact 1-4 pair) */
  int32_t i, j;
  float charge_product;           /* e^2 */
  float sigma;                    /* Å */
  float epsilon;                  /* kcal/mol */
} prismq_exception;

typedef struct prismq_hcluster {  /* input.rs:625 HCluster */
  int32_t central_atom;
  int32_t hydrogen_atoms[3];      /* -1 for unused slots */
  float bond_lengths[3];
  int32_t n_hydrogens;            /* 1..3 */
  float inv_mass_central;
  float inv_mass_h;
} prismq_hcluster;

typedef struct prismq_topology {
  int32_t n_atoms;
  const float* positions;         /* [3N] Å */
  const float* masses;            /* [N] amu, already repartitioned (HMR) */
  const float* charges;           /* [N] e */
  const float* lj_sigma;          /* [N] Å */
  const float* lj_epsilon;        /* [N] kcal/mol */
  int32_t n_bonds;       const prismq_bond* bonds;
  int32_t n_angles;      const prismq_angle* angles;
  int32_t n_dihedrals;   const prismq_dihedral* dihedrals;
  int32_t n_exceptions;  const prismq_exception* exceptions;
  /* Exclusions per atom (CSR over atoms): every partner whose ordinary
   * nonbonded pair is removed (1-2, 1-3 and the 1-4 pairs that carry an
   * exception).  input.rs:1094 `exclusions: Vec<Vec<usize>>`. */
  const int32_t* exclusion_offsets;  /* [N+1] */
  const int32_t* exclusions;         /* [exclusion_offsets[N]] */
  int32_t n_clusters;    const prismq_hcluster* clusters;
} prismq_topology;

/* ---- run parameters (engine defaults: fused_engine.rs:13278-13366, set_dt :15342) ---- */

typedef enum prismq_nlist_mode {
  PRISMQ_NLIST_COMPLETE = 0,  /* every pair with r^2 <= r_list^2 (brute-force equal) */
  PRISMQ_NLIST_REF27 = 1      /* reference scheme: fixed 10 Å grid from the initial box,
                                 27-cell stencil, r^2 <= 144 (nhs_neighbor_warp.cuh:10-121) */
} prismq_nlist_mode;

typedef struct prismq_params {
  float dt;                   /* ps; 0.004 under HMR */
  float temperature;          /* K */
  float gamma;                /* ps^-1 (0 => Hamiltonian kicks, no OU noise) */
  float cutoff;               /* Å, 10 */
  float skin;                 /* Å, list radius = cutoff + skin */
  int32_t rebuild_interval;   /* steps; a half-skin displacement trigger also rebuilds */
  int32_t com_interval;       /* steps between COM-velocity removals (100; 0 = never) */
  int32_t max_constraint_iter;/* SHAKE/RATTLE iteration bound (100) */
  uint32_t seed;              /* Philox key word 0 */
  uint32_t stream;            /* Philox key word 1 (system id in a batch) */
  float shake_tol;            /* SHAKE: |r^2 - L^2| / L^2 (shake_cluster_positions :1890, 1e-4; <= 0 selects it) */
  float rattle_tol;           /* RATTLE: |r·v_rel| / (|r| max(|v_rel|, 1)) (:2176, 1e-5; <= 0 selects it) */
  int32_t constraint_check_fp64; /* 1: constraint residuals and multipliers in FP64 (0: FP32 as the reference) */
  int32_t precision;          /* prismq_precision of the run */
} prismq_params;

typedef enum prismq_precision {
  PRISMQ_PRECISION_FP32 = 0,  /* production: FP32 math, int64 fixed-point forces */
  PRISMQ_PRECISION_FP64 = 1   /* precision study: FP64 state, forces and integrator everywhere */
} prismq_precision;

/* Fill *p with the reference engine defaults under HMR
 * (dt 0.004, T 300, γ 1, cutoff 10, skin 2, rebuild 20, COM 100, 100 iterations,
 * SHAKE 1e-4, RATTLE 1e-5, FP32 constraint checks, FP32 precision). */
void prismq_params_default(prismq_params* p);

const char* prismq_last_error(void);
int prismq_abi_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int prismq_device_count(void);
/* Kernels this library has launched in this process (graph nodes counted). */
long long prismq_kernel_launches(void);
/* The CUDA runtime is linked into this library, so its current device is its
 * own: another framework's device selection (torch.cuda.set_device, ...) does
 * not reach it.  A process that drives GPU k calls prismq_set_device(k) before
 * it creates systems, batches or servers; handles live on the device that was
 * current on the thread that created them and are used from threads that have
 * the same device selected (a server's worker thread takes its creator's).
 * No counterpart in the reference (one engine per process and stream).
 * Applies to the calling thread. */
prismq_status prismq_set_device(int32_t ordinal);
/* The calling thread's current device in this library (-1 without a device). */
int32_t prismq_device_ordinal(void);
/* out = {ordinal, streaming multiprocessors, peak SM clock in kHz} of the
 * calling thread's current device. */
prismq_status prismq_device_info(int32_t out[3]);

/* ---- synthetic poly-alanine-like systems (host only, no GPU) ---- */

typedef struct prismq_topology_buf prismq_topology_buf;

/* Build n_chains seeded chains of n_residues each (10 atoms/residue: N H CA HA
 * CB HB1 HB2 HB3 C O; ff14SB ALA charges/LJ/bonded terms; exact 1-4
 * exceptions qq/1.2, σ̄, ε̄/2; HMR with hydrogen mass 3.024 amu).
 * Each chain grows inside its own region: a sphere of atom density `density`
 * (atoms/Å^3; <= 0 selects 0.03) when box_edge <= 0, otherwise one cell of a
 * box of edge box_edge split among the chains.  Self-avoiding growth with
 * ideal internal coordinates stalls above ~0.035 atoms/Å^3, so a region that
 * is too dense is enlarged by 5% per attempt.  Deterministic for a given
 * seed, with identical bits on x86-64 and aarch64. */
prismq_status prismq_polyala_build(int32_t n_chains, int32_t n_residues, uint64_t seed,
                                   float density, float box_edge,
                                   prismq_topology_buf** out);
/* The same chains collapsed into compact systems, the synthetic inputs of the
 * benchmark configurations (a random-walk backbone collapsed into a globule;
 * chains packed without overlap in a cube).  The chains are grown at
 * 0.02 atoms/Å^3 and then squeezed by a deterministic relaxation: bond and
 * angle restraints from the topology, a contact distance of
 * max(0.8 (Rmin_i/2 + Rmin_j/2), 2 Å) between atoms more than three bonds
 * apart, and a region that shrinks to its target:
 *   box_edge <= 0: one sphere per chain holding it at `density` atoms/Å^3
 *                  (<= 0 selects 0.0746: 2,500 atoms in a 40 Å globule);
 *   box_edge  > 0: one cube of edge box_edge holding every chain.
 * Hydrogens end on their constraint lengths.  stats (may be NULL) receives:
 * relaxation iterations, the largest remaining contact overlap (Å), the
 * largest distance of an atom outside its region (Å), and the closest pair
 * of atoms more than three bonds apart (Å).  Deterministic for a given seed,
 * with identical bits on x86-64 and aarch64. */
prismq_status prismq_polyala_build_compact(int32_t n_chains, int32_t n_residues, uint64_t seed,
                                           float density, float box_edge, double stats[4],
                                           prismq_topology_buf** out);
/* View the arrays of a built topology; valid until prismq_topology_free. */
prismq_status prismq_topology_view(const prismq_topology_buf* buf, prismq_topology* out);
void prismq_topology_free(prismq_topology_buf* buf);

/* ---- PRISM-PREP topology JSON (host only, no GPU) ----
 *
 * Replaces PrismPrepTopology::load (crates/prism-nhs/src/input.rs:1972),
 * validate (:1996-2290), lower_harmonic_parameters (:467-520),
 * validate_for_nonbonded_execution (:1429-1450) and apply_hmr (:2482-2560):
 * the JSON a PRISM-PREP run writes becomes a prismq_topology ready for
 * prismq_system_create / prismq_batch_add_system.
 *   - Bond and angle force constants are lowered from the file's
 *     harmonic_parameter_contract convention to U = k (x - x0)^2
 *     (OPENMM_FULL_K_HALF_ENERGY: k x 0.5 in binary64, then float32).
 *     The contract's canonical SHA-256 is checked.
 *   - Strict exclusions come from `exclusions`; exact 1-4 pairs from
 *     `nonbonded_exceptions`, whose completeness contract (counts and both
 *     SHA-256 digests) is checked.
 *   - Hydrogen mass repartitioning runs unless the file records
 *     hmr_applied = true. */
typedef struct prismq_prep_options {
  int32_t apply_hmr;                 /* 1: repartition unless the file records it done (default 1) */
  int32_t require_harmonic_contract; /* 1: refuse a file without harmonic_parameter_contract (default 1);
                                        0: cast its coefficients to float32 unscaled */
  int32_t require_exceptions;        /* 1: NonbondedExecutionPolicy::RequireExactV2 (default 1) */
  int32_t reserved;
  double hmr_factor;                 /* hydrogen mass multiplier (default 3.0) */
} prismq_prep_options;

typedef struct prismq_prep_report {
  int32_t hmr_performed;             /* 1 if repartitioning ran during this load */
  int32_t n_repartitioned;           /* clusters repartitioned */
  int32_t n_skipped;                 /* clusters left alone (central atom would fall below 1 amu) */
  int32_t exact_exceptions;          /* number of exact 1-4 exception pairs */
  double bond_scale, angle_scale;    /* source / target energy prefactor applied to k */
  double total_mass_before, total_mass_after;  /* cluster masses, amu (binary64) */
} prismq_prep_report;

void prismq_prep_options_default(prismq_prep_options* opt);
/* Parse `len` bytes of UTF-8 JSON.  opt and report may be NULL (defaults; no report).
 * PRISMQ_E_INVALID with prismq_last_error() naming the first violated rule. */
prismq_status prismq_topology_from_prep_json(const char* text, size_t len, const prismq_prep_options* opt,
                                             prismq_topology_buf** out, prismq_prep_report* report);
/* Same, reading a file; PRISMQ_E_NOT_FOUND if it cannot be opened. */
prismq_status prismq_topology_load_prep_json(const char* path, const prismq_prep_options* opt,
                                             prismq_topology_buf** out, prismq_prep_report* report);

/* ---- single system (the drop-in for NhsAmberFusedEngine, fused_engine.rs:6554) ---- */

typedef struct prismq_system prismq_system;

/* NhsAmberFusedEngine::new_on_stream (fused_engine.rs:10800): validate and
 * lower the topology (exception CSR :11625-11700, incidence :11704-11745,
 * H clusters :11827-11938, cell grid :12285-12330), upload, and initialise
 * Maxwell–Boltzmann velocities at params->temperature with COM removed. */
prismq_status prismq_system_create(const prismq_topology* topo, const prismq_params* params,
                                   prismq_system** out);
void prismq_system_destroy(prismq_system* sys);
int32_t prismq_system_n_atoms(const prismq_system* sys);

/* set_dt (fused_engine.rs:15342) and friends; take effect at the next step. */
prismq_status prismq_set_dt(prismq_system* sys, float dt);
prismq_status prismq_set_temperature(prismq_system* sys, float temperature);
prismq_status prismq_set_gamma(prismq_system* sys, float gamma);

/* Host AoS float[3N] in/out (get_positions :24117, get_velocities :20939). */
prismq_status prismq_set_positions(prismq_system* sys, const float* xyz);
prismq_status prismq_set_velocities(prismq_system* sys, const float* vxyz);
prismq_status prismq_get_positions(prismq_system* sys, float* xyz);
prismq_status prismq_get_velocities(prismq_system* sys, float* vxyz);
/* Step counter (the value of `timestep` before the next step). */
prismq_status prismq_get_step(prismq_system* sys, int64_t* step);
prismq_status prismq_set_step(prismq_system* sys, int64_t step);

/* ---- run protocol: per-step temperature, friction and timestep ----
 *
 * Replaces ProtocolState (protocol_state.cuh:14-62), its constructor
 * ProtocolState::from_cryo_uv (protocol_state.rs:602-700), the director's
 * per-step evaluation (protocol_director.cu:54-143) and
 * NhsAmberFusedEngine::set_cryo_uv_protocol (fused_engine.rs:18815),
 * compute_cryo_friction (:15366-15396) and set_adaptive_dt (:13986).
 * The device evaluates the protocol at the start of every step inside the
 * captured step graph (no extra launch); each system of a batch carries its
 * own.  Step k after installation (k = 0, 1, ...) uses director step
 * current_step + 1 + k.  UV bursts, wavelength scans and steering hints are
 * not part of the MD step and are not carried. */
typedef struct prismq_protocol {
  float start_temp, end_temp;          /* K: cold and warm temperatures */
  int32_t cold_hold_steps, ramp_steps, warm_hold_steps, ramp_down_steps, cold_return_steps;
  float gamma_base;                    /* ps^-1 after equilibration */
  int32_t cryo_enabled;                /* 1: γ x sqrt(300 / max(T, 10)) below 300 K */
  int32_t equilibration_steps;         /* director steps of the friction blend (10000) */
  float equilibration_gamma;           /* ps^-1 at the start of the blend (1000) */
  int32_t adaptive_dt;                 /* 0: base_dt; 1: holds base_dt, ramps base_dt/2;
                                          2: holds 1.5 base_dt, ramps base_dt */
  float base_dt;                       /* ps */
  int32_t current_step;                /* director step at installation (0) */
} prismq_protocol;

/* Physiological protocol: 300 K throughout, γ 1 ps^-1 after the reference's
 * 10000-step equilibration blend from 1000 ps^-1, dt 0.004 ps, no cryo or
 * adaptive dt. */
void prismq_protocol_default(prismq_protocol* p);
/* The protocol's values at one director step: out = {T (K), γ (ps^-1), dt (ps)}. */
prismq_status prismq_protocol_eval(const prismq_protocol* p, int64_t director_step, float out[3]);
/* Install a protocol (NULL removes it; the system keeps its current T, γ, dt).
 * While one is installed, set_temperature / set_gamma return PRISMQ_E_INVALID
 * and set_dt sets its base_dt. */
prismq_status prismq_set_protocol(prismq_system* sys, const prismq_protocol* p);
/* {T, γ, dt} the next step will use. */
prismq_status prismq_get_step_params(prismq_system* sys, float out[3]);

/* ---- checkpoints: the dynamic state of one system at a step boundary ----
 *
 * Replaces the MD part of capture_process_checkpoint_fields /
 * restore (fused_engine.rs:24718-25772): positions, velocities, the step
 * counter, the neighbour-list schedule (steps since the last build, the
 * positions of that build), the run parameters and the protocol.  A restored
 * system continues bit for bit as the saved one would have: noise is
 * counter-based, and rows rebuilt from the saved list-build positions give
 * the same forces.  The blob is self-describing (magic, version, a topology
 * fingerprint and a payload checksum); restore refuses a blob of another
 * topology, size or library version, and a damaged one.  FP32 systems. */
prismq_status prismq_checkpoint_size(prismq_system* sys, size_t* bytes);
/* The same size for a system of n_atoms atoms (host only: sizes a buffer
 * before the system exists, e.g. a served job's snapshot_out). */
prismq_status prismq_checkpoint_size_for_atoms(int64_t n_atoms, size_t* bytes);
prismq_status prismq_checkpoint_save(prismq_system* sys, void* buf, size_t cap, size_t* written);
prismq_status prismq_checkpoint_restore(prismq_system* sys, const void* buf, size_t len);

/* ---- trajectory frames (the reference records none: D-FRAMES-NOT-CAPTURED) ----
 *
 * Every `interval` steps the state at that step boundary (positions after the
 * step's drift and SHAKE, velocities after its post-force phases; the values
 * prismq_get_positions / get_velocities return there) is copied device to
 * device into a ring of `capacity` frames: a step() call runs in segments
 * that end on the frame boundaries, which changes no result.
 * interval 0 stops recording and frees the ring.  prismq_frames_read copies
 * out, oldest first, up to max_frames frames not yet read: AoS float[3N] per
 * frame into xyz (and vxyz when velocities were requested; may be NULL), the
 * boundary step of each into steps (may be NULL).  *dropped counts frames
 * overwritten before they were read.  FP32 systems. */
prismq_status prismq_frames_configure(prismq_system* sys, int32_t interval, int32_t capacity, int32_t with_velocities);
prismq_status prismq_frames_read(prismq_system* sys, float* xyz, float* vxyz, int64_t* steps, int32_t max_frames,
                                 int32_t* n_out, int64_t* dropped);

/* Force evaluation at the current positions (FORCE_N phase, nhs_amber_fused.cu:2993-3484).
 * pe_total: FP64 total potential energy (may be NULL).
 * f_aos: float[3N] kcal/mol/Å (may be NULL).  f_fixed: int64[3N] at 2^-32 (may be NULL). */
prismq_status prismq_compute_forces(prismq_system* sys, double* pe_total, float* f_aos,
                                    int64_t* f_fixed);
/* Energy components: [bond, angle, dihedral, exception, nonbonded(shifted), kinetic]. */
prismq_status prismq_energy_components(prismq_system* sys, double out[6]);
/* Virial tensor W_ab = Σ_i x_a F_b (kcal/mol, row-major [9]) at the current
 * positions, reduced in FP64. */
prismq_status prismq_virial(prismq_system* sys, double out[9]);
/* FP64 state and forces (FP64 systems hold them natively; FP32 systems return
 * their FP32 values widened).  double[3N] each; forces at the last evaluation. */
prismq_status prismq_get_state_f64(prismq_system* sys, double* xyz, double* vxyz);
prismq_status prismq_get_forces_f64(prismq_system* sys, double* f);

/* Build the pair list at the current positions and return the canonical
 * (i<j) pairs, sorted, as int32 pairs_out[2*n].  REF27 reproduces the
 * reference pair set (exclusion CSR = exclusions minus exception pairs);
 * COMPLETE returns every pair with r^2 <= (cutoff+skin)^2 in the same FP32
 * arithmetic.  *n receives the number of pairs; PRISMQ_E_CAPACITY if
 * cap < n (n still reported). */
prismq_status prismq_build_neighbors(prismq_system* sys, prismq_nlist_mode mode,
                                     int32_t* pairs_out, size_t cap, size_t* n);

/* Advance n_steps MD steps (step(), fused_engine.rs:18963, phase order
 * MD_EXECUTION_PHASES :6223-6235 plus the post-step clamp/RATTLE :17498-17800). */
prismq_status prismq_step(prismq_system* sys, int64_t n_steps);

/* Debug entry points used by the parity tests (single phases on the device). */
typedef enum prismq_phase_set {
  PRISMQ_PHASES_PRE = 1,   /* OU½ → RATTLE → KICK½ → RATTLE → DRIFT → SHAKE */
  PRISMQ_PHASES_POST = 2   /* KICK½ → RATTLE → OU½ → velocity clamp → RATTLE */
} prismq_phase_set;
/* Run one phase set with the current forces, using noise for step `step`. */
prismq_status prismq_debug_phases(prismq_system* sys, prismq_phase_set set, int64_t step);
/* Host copy of the injected noise: three normals per atom for (seed, stream,
 * atom, step, purpose) — bit-identical to what the kernels draw. */
void prismq_debug_noise(uint32_t seed, uint32_t stream, uint32_t atom, uint64_t step,
                        uint32_t purpose, float out3[3]);

/* ---- batch: many independent systems advanced together ---- */

typedef struct prismq_batch prismq_batch;

/* Create an empty batch with room for max_atoms atoms in total. */
prismq_status prismq_batch_create(int64_t max_atoms, int32_t max_systems, prismq_batch** out);
/* Same, for systems of one precision (prismq_precision); every system added
 * must carry params.precision equal to it. */
prismq_status prismq_batch_create_ex(int64_t max_atoms, int32_t max_systems, int32_t precision,
                                     prismq_batch** out);
void prismq_batch_destroy(prismq_batch* b);
/* Admit a system; *slot receives its index.  PRISMQ_E_CAPACITY if it does not fit. */
prismq_status prismq_batch_add_system(prismq_batch* b, const prismq_topology* topo,
                                      const prismq_params* params, int32_t* slot);
prismq_status prismq_batch_remove_system(prismq_batch* b, int32_t slot);
/* Advance every resident system by n_steps (one captured CUDA graph per step). */
prismq_status prismq_batch_step(prismq_batch* b, int64_t n_steps);
prismq_status prismq_batch_get_state(prismq_batch* b, int32_t slot, float* xyz, float* vxyz);
prismq_status prismq_batch_set_state(prismq_batch* b, int32_t slot, const float* xyz,
                                     const float* vxyz);
prismq_status prismq_batch_get_step(prismq_batch* b, int32_t slot, int64_t* step);
prismq_status prismq_batch_status(prismq_batch* b, int32_t slot);
/* Run protocol of one resident system (see prismq_set_protocol). */
prismq_status prismq_batch_set_protocol(prismq_batch* b, int32_t slot, const prismq_protocol* p);
prismq_status prismq_batch_get_step_params(prismq_batch* b, int32_t slot, float out[3]);
/* Checkpoint of one resident system (see prismq_checkpoint_save); a blob
 * saved from a single system restores into a batch slot holding the same
 * topology, and the other way round. */
prismq_status prismq_batch_checkpoint_size(prismq_batch* b, int32_t slot, size_t* bytes);
prismq_status prismq_batch_checkpoint_save(prismq_batch* b, int32_t slot, void* buf, size_t cap, size_t* written);
prismq_status prismq_batch_checkpoint_restore(prismq_batch* b, int32_t slot, const void* buf, size_t len);
/* Trajectory frames of one resident system (see prismq_frames_configure). */
prismq_status prismq_batch_frames_configure(prismq_batch* b, int32_t slot, int32_t interval, int32_t capacity,
                                            int32_t with_velocities);
prismq_status prismq_batch_frames_read(prismq_batch* b, int32_t slot, float* xyz, float* vxyz, int64_t* steps,
                                       int32_t max_frames, int32_t* n_out, int64_t* dropped);
/* Layout of the production neighbour list (FP32 systems in complete mode):
 *   0 (default) one row of partner indices per atom (at most 1024), the
 *     layout REF27 and FP64 runs always use;
 *   1 cluster-pair tiles: i-clusters of 8 consecutive atoms against
 *     j-clusters of 4, one {j-cluster, 32-bit pair mask} per tile, the tiles
 *     of an i-cluster in ascending j-cluster order (at most 768).
 * The pair set is the same; the forces differ only in the grouping of their
 * FP32 partial sums, and each layout is bit-reproducible on its own.  Setting
 * it rebuilds every resident system's list before the next step, so set it
 * before stepping.  No counterpart in the reference, which keeps one full
 * row per atom (nhs_neighbor_warp.cuh:10-121). */
prismq_status prismq_batch_set_pair_layout(prismq_batch* b, int32_t layout);
int32_t prismq_batch_pair_layout(const prismq_batch* b);
prismq_status prismq_set_pair_layout(prismq_system* sys, int32_t layout);
/* The autotuner's choice for the batch's force kernel: out[0] = variant
 * (-1 before the first step), out[1] = threads per block (four per atom: 128
 * for 32 atoms, 256 for 64), out[2] = minimum resident blocks per SM given to
 * the register allocator.  The launch shape does not change results. */
prismq_status prismq_batch_tuning(prismq_batch* b, int32_t out[3]);
/* The same with out[3] = atoms per block and out[4] = how many row-index
 * iterations ahead the kernel asks L2 for the atom's row (0: no prefetch).
 * No counterpart in the reference (its launch shape is fixed, one thread per
 * atom, fused_engine.rs:19268-19350). */
prismq_status prismq_batch_tuning_ex(prismq_batch* b, int32_t out[5]);
/* Pin the force kernel's launch shape to `variant` (0 .. n-1; *n_variants
 * receives n, may be NULL), or hand the choice back to the autotuner with
 * variant -1.  Every shape gives the same bits. */
prismq_status prismq_batch_set_force_variant(prismq_batch* b, int32_t variant, int32_t* n_variants);
/* out[0] = steps taken, out[1] = neighbour-list builds so far. */
prismq_status prismq_batch_counters(prismq_batch* b, int32_t slot, int64_t out[2]);
prismq_status prismq_batch_energy(prismq_batch* b, int32_t slot, double out[6]);
prismq_status prismq_batch_virial(prismq_batch* b, int32_t slot, double out[9]);
prismq_status prismq_batch_get_state_f64(prismq_batch* b, int32_t slot, double* xyz, double* vxyz);
prismq_status prismq_batch_get_forces_f64(prismq_batch* b, int32_t slot, double* f);
int64_t prismq_batch_resident_atoms(const prismq_batch* b);
/* Whole-arena state transfer: float[3*span] in arena atom order (span =
 * prismq_batch_atom_span; system `slot` starts at prismq_batch_atom_offset).
 * Entries of free arena ranges are ignored on upload.  Uploaded positions that
 * differ bitwise from the resident ones refresh that system's list and forces
 * before its next step.  Pinned (page-locked) host arrays are read and written
 * by the transfer kernel directly over the host link; pageable arrays go
 * through a device staging copy.  get_state_all returns with the arrays
 * filled.  set_state_all is ordered before every later call on the batch;
 * a pageable array may be reused when it returns, a pinned one once a later
 * call that returns host data (get_state_all, ...) has returned. */
int64_t prismq_batch_atom_span(const prismq_batch* b);
int64_t prismq_batch_atom_offset(const prismq_batch* b, int32_t slot);
prismq_status prismq_batch_set_state_all(prismq_batch* b, const float* xyz, const float* vxyz);
prismq_status prismq_batch_get_state_all(prismq_batch* b, float* xyz, float* vxyz);
/* A host-driven step in one call: set_state_all(xyz_in, vxyz_in), n_steps
 * steps, get_state_all(xyz_out, vxyz_out), enqueued back to back with one
 * wait at the end (any array may be NULL; n_steps 0 only transfers).  With
 * a pinned xyz_out the positions are copied back while the last step's forces
 * and post-force phases still run (those phases move only velocities).  The
 * outputs are filled even when a system fails; the return value is then
 * that failure, as from prismq_batch_step. */
prismq_status prismq_batch_step_host(prismq_batch* b, int64_t n_steps, const float* xyz_in, const float* vxyz_in,
                                     float* xyz_out, float* vxyz_out);
/* Advance every resident system by n_steps+1 steps, of which n_steps are
 * captured in one CUDA graph and timed on the device: total_ms covers those
 * n_steps; phase_ms (optional, 5*n_steps entries) holds, for step i at
 * [5i..5i+4], the device time on the main stream of (decision + control +
 * OU normals), row builder, rebuilt systems' forces up to the join,
 * integrate, and then the other systems' force launch on the second stream,
 * which overlaps the first three (events recorded between the launches). */
prismq_status prismq_batch_run_timed(prismq_batch* b, int64_t n_steps, float* total_ms, float* phase_ms);
/* Average device time of the force kernel over every resident system,
 * launched alone n times on the main stream (the roofline's denominator). */
prismq_status prismq_batch_time_force(prismq_batch* b, int32_t n_launches, float* ms_per_launch);
int32_t prismq_batch_resident_systems(const prismq_batch* b);

/* ---- job server: continuous batching of independent MD jobs ----
 *
 * The reference has no batched or served form of this path (its parallel
 * replica entry points bail out, fused_engine.rs:18306 and :18433); a caller
 * runs one NhsAmberFusedEngine per system (new_on_stream :10800, run :23911,
 * get_positions :24117).  The server replaces that loop: one worker thread owns
 * a batch arena sized from max_hbm_bytes, admits queued jobs whenever their
 * atoms and terms fit in the free arena ranges (admission by HBM footprint),
 * advances every resident job together in chunks of at most chunk_steps steps
 * (each chunk ends exactly where the nearest job finishes), and retires
 * finished jobs between chunks.  A job's trajectory depends only on its own
 * topology and params, never on which other jobs share the GPU: results are
 * bit-identical to running the job alone.
 *
 * Snapshots: a job may start from a checkpoint (resume: the bytes of
 * prismq_checkpoint_save or of another job's snapshot, same topology) and may
 * ask for its final checkpoint (snapshot_out, snapshot_cap >=
 * prismq_checkpoint_size_for_atoms).  A long run split into jobs chained
 * through snapshots is bit-identical to the run in one job; a job refused
 * at restore fails with the restore's status and message.
 *
 * Threading: every prismq_server_* call is internally locked and may come
 * from any thread. */

typedef struct prismq_server prismq_server;

typedef struct prismq_server_config {
  int32_t max_systems;  /* resident jobs at most (<= 0 selects 1024) */
  int32_t chunk_steps;  /* steps between scheduling points (<= 0 selects 50) */
  double max_bypass_s;  /* how long later jobs may overtake a queued job that does
                           not fit yet (< 0 selects 1.0; 0 = strict FIFO) */
} prismq_server_config;

typedef struct prismq_job {
  const prismq_topology* topology; /* validated and copied by submit */
  prismq_params params;            /* seed/stream select the job's noise */
  int64_t n_steps;                 /* >= 1 */
  float* positions_out;            /* host float[3N] or NULL: final positions */
  float* velocities_out;           /* host float[3N] or NULL: final velocities */
  uint64_t tag;                    /* echoed in the result */
  const struct prismq_protocol* protocol; /* NULL: constant T, γ, dt; else copied by submit */
  const void* resume;              /* NULL, or a checkpoint of this topology to start from (copied by submit) */
  size_t resume_len;
  void* snapshot_out;              /* NULL, or a host buffer for the job's final checkpoint */
  size_t snapshot_cap;             /* its size (prismq_checkpoint_size of the system) */
} prismq_job;

typedef struct prismq_job_result {
  int64_t job_id;
  uint64_t tag;
  prismq_status status;  /* PRISMQ_OK, or why the job stopped */
  int32_t n_atoms;
  int64_t steps_done;
  double submit_s;  /* server clock (seconds since create) at submit */
  double start_s;   /* admission into the arena */
  double end_s;     /* results written to the job's buffers */
  char message[160];
  uint64_t snapshot_len;  /* bytes written to snapshot_out (0: none requested, or the job failed) */
} prismq_job_result;

typedef struct prismq_server_stats {
  int64_t submitted, completed, failed, queued, resident_jobs, resident_atoms;
  int64_t capacity_atoms;  /* arena atom capacity */
  int64_t device_bytes;    /* device memory held by the arena */
  int64_t chunks;          /* batch step calls so far */
  double atom_steps;       /* atom-steps completed by all jobs */
  double busy_s;           /* worker time inside batch steps */
  double uptime_s;
} prismq_server_stats;

void prismq_server_config_default(prismq_server_config* cfg);
/* Reserve an arena of at most max_hbm_bytes device bytes and start the
 * worker.  cfg may be NULL (defaults). */
prismq_status prismq_server_create(int64_t max_hbm_bytes, const prismq_server_config* cfg,
                                   prismq_server** out);
/* Validate and queue a job; *job_id receives its id.  PRISMQ_E_CAPACITY if the
 * job could never fit in the arena.  The job's output buffers must stay valid
 * until its result has been polled. */
prismq_status prismq_server_submit(prismq_server* s, const prismq_job* job, int64_t* job_id);
/* Move up to cap finished results into out (completion order); waits up to
 * wait_ms for at least one when none is ready.  *n receives the count. */
prismq_status prismq_server_poll(prismq_server* s, prismq_job_result* out, int32_t cap, int32_t* n,
                                 int32_t wait_ms);
prismq_status prismq_server_stats_get(prismq_server* s, prismq_server_stats* out);
/* Stop the worker after its current chunk; queued and resident jobs are
 * dropped without results. */
void prismq_server_destroy(prismq_server* s);

/* ---- neighbour rows without device allocation ----
 *
 * No counterpart in the reference: it serves callers that cannot allocate
 * device memory while they run — for example a serving process that reserves
 * its whole HBM budget for job arenas at start-up, or a host loop whose
 * allocator policy forbids cudaMalloc/cudaFree after start-up because they
 * synchronise the device and fragment memory.
 *
 * Builds the complete neighbour rows of a point set (every j != i with
 * (dx*dx + dy*dy) + dz*dz <= list_radius^2 in FP32, the batched builder's
 * complete-mode rule) into caller-owned DEVICE buffers:
 *   d_xyz     device float[3*n_atoms] positions (Å)
 *   d_rows    device int32[n_atoms*row_cap]; row i holds its neighbours
 *   d_counts  device int32[n_atoms]; row lengths (-1 for a row that overflowed)
 *   stream    a cudaStream_t (NULL for the default stream)
 * Limits: 1 <= n_atoms <= 65536 and 1 <= row_cap <= 1024, checked on the host
 * and rejected with PRISMQ_E_CAPACITY before any GPU work.  Two limits are
 * found on the GPU and reported after the work: a cell (cells are at least
 * list_radius/2 wide) holding more than 512 atoms returns
 * PRISMQ_E_CELL_OVERFLOW with every count set to -1, and a row longer than
 * row_cap returns PRISMQ_E_NEIGHBOR_OVERFLOW with that row's count set to -1
 * (nothing is written past row_cap; the other rows are complete).  The call
 * calls no cudaMalloc or cudaFree: its cell lists live in one fixed file-scope
 * device array (about 0.8 MB) that every GPU loading the library keeps until
 * the process exits.  The first call on a device looks up that array's device
 * address (set-up work; make it before any stream capture); the address is
 * kept for the process, so the entry point must not be used across a
 * cudaDeviceReset.  Every call reuses the same array, so calls that overlap on
 * the GPU race and must be serialised by the caller.  The call synchronises
 * the stream: it returns after the stream has finished the work. */
prismq_status prismq_neighbor_rows_noalloc(const float* d_xyz, int32_t n_atoms, float list_radius,
                                           int32_t row_cap, int32_t* d_rows, int32_t* d_counts,
                                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PRISMQ_MD_H */
