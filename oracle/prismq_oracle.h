/*
 * CPU oracle for the Prism-Q classical MD step — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm (Delfictus/Prism-Q,
 * crates/prism-gpu/src/kernels/nhs_amber_fused.cu, nhs_neighbor_warp.cuh,
 * housekeeping.cu and crates/prism-nhs/src/fused_engine.rs), used only by the
 * tests, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
 * baseline leg.  The product library never links or calls it.
 *
 * Parity pins (see tests/): the neighbour scheme is pinned against the
 * reference's own CPU check scripts/physics_refs/neighbor_list.py through
 * committed golden vectors (synthetic_600: 94,216 brute-force pairs, 93,912
 * kept, 304 missed); Philox4x32-10 against the Random123 known-answer vectors
 * quoted in scripts/physics_refs/rng_streams.py:87-92; the 418.4 half-kick
 * against fused_engine.rs:4723-4731.
 */
#ifndef PRISMQ_ORACLE_H
#define PRISMQ_ORACLE_H

#include <stdint.h>

#include "../include/prismq_md.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  float dt, temperature, gamma, cutoff;
  float c1;            /* exp(-gamma*dt/2), supplied so both sides use the same float */
  int max_iter;        /* SHAKE/RATTLE iteration bound */
  int com_interval;    /* 0 = never */
  uint32_t seed, stream;
} orc_params;

typedef struct orc_sys orc_sys;

/* ---- random numbers ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_normal3(uint32_t seed, uint32_t stream, uint32_t atom, uint64_t step, uint32_t purpose,
                 float out[3]);

/* ---- neighbour schemes (pairs i<j written to out[2*k], returns count or -needed) ---- */
/* The reference cell scheme: grid fixed from `grid_pos` (the construction-time
 * positions), 10 Å cells, truncation + clamp, 27-cell stencil, keep !(r2 > r2max). */
long orc_pairs_ref27(int n, const float* pos, const float* grid_pos, float r2max,
                     const int32_t* excl_off, const int32_t* excl, int32_t* out, long cap,
                     int* max_occupancy);
/* Every pair with !(r2 > r2max) in the same FP32 arithmetic. */
long orc_pairs_brute(int n, const float* pos, float r2max, const int32_t* excl_off,
                     const int32_t* excl, int32_t* out, long cap);

/* ---- systems ---- */
orc_sys* orc_create(const prismq_topology* t, const orc_params* p);
void orc_destroy(orc_sys* s);
int orc_n_atoms(const orc_sys* s);
void orc_set_state(orc_sys* s, const float* x, const float* v);
void orc_get_state(const orc_sys* s, float* x, float* v);
/* The ordinary-pair exclusion CSR the reference uploads (exclusions minus
 * exception pairs), for comparison with the library's parity output. */
int orc_ref_exclusions(const orc_sys* s, int32_t* off, int32_t* list, long cap);

/* FP32 restatement of the reference force phase (per-atom gather, full
 * ascending neighbour rows from the REF27 scheme at the current positions,
 * pairs14 scan per neighbour, exact exceptions).  f: float[3N].
 * e5: bond, angle, dihedral, exception, nonbonded (shifted) in FP64. */
int orc_forces_ref_f32(orc_sys* s, float* f, double* e5, int threads);
/* FP64 oracle: the same pair set (FP32 r2 = fmaf(dz,dz,fmaf(dy,dy,dx*dx)),
 * r2 < cutoff^2 and >= 0.01, exclusions and exception pairs removed), all
 * arithmetic in double. */
int orc_forces_f64(orc_sys* s, double* f, double* e5, int threads);
int orc_forces_f64_rule(orc_sys* s, double* f, double* e5, int threads, int incl64);
int orc_rattle_all(orc_sys* s);
int orc_shake_all(orc_sys* s, const float* xs);
void orc_kick_all(orc_sys* s, const float* f);
void orc_clamp_all(orc_sys* s);
void orc_ou_all(orc_sys* s, const float* z, float c1);
void orc_term_forces(const orc_sys* s, float* fb, float* fa, float* fd);

/* Integrator phase sets on the current state with forces given as int64
 * fixed point (2^-32 kcal/mol/Å).  set 1 = OU½, RATTLE, KICK½, RATTLE, DRIFT,
 * SHAKE; set 2 = KICK½, RATTLE, OU½, clamp, RATTLE.  Returns 0 or an error
 * code (1 SHAKE, 2 RATTLE). */
int orc_phases(orc_sys* s, int set, const int64_t* f_fixed, long long step);
/* Run protocol: out = {T, gamma, dt, c1} at one director step; with a protocol
 * installed every step st uses director step st - origin. */
void orc_protocol_eval(const prismq_protocol* p, long long director_step, float out[4]);
void orc_set_protocol(orc_sys* s, const prismq_protocol* p, long long origin);
/* COM velocity removal (exact int64 Σ m·v, double Σ m). */
void orc_com_remove(orc_sys* s);

/* The reference step loop on the CPU (the reported baseline): per step
 * FORCE_N, OU½, RATTLE, KICK½, RATTLE, DRIFT, SHAKE, neighbour rebuild,
 * FORCE_NP1, KICK½, RATTLE, OU½, clamp, RATTLE; COM removal every
 * com_interval steps.  Forces are the FP32 restatement.  Returns 0 or error. */
int orc_run(orc_sys* s, long n_steps, int threads);
long long orc_step_count(const orc_sys* s);

#ifdef __cplusplus
}
#endif
#endif
