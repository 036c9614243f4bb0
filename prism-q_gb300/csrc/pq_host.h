// Host-side structures shared by the topology builder and the engine.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/prismq_md.h"

namespace pq {

// Owned copy of a prismq_topology (the builder's output, or a caller's input
// after validation).
struct HostTopology {
  int32_t n_atoms = 0;
  std::vector<float> positions, masses, charges, lj_sigma, lj_epsilon;
  std::vector<prismq_bond> bonds;
  std::vector<prismq_angle> angles;
  std::vector<prismq_dihedral> dihedrals;
  std::vector<prismq_exception> exceptions;
  std::vector<int32_t> exclusion_offsets, exclusions;
  std::vector<prismq_hcluster> clusters;

  void view(prismq_topology* t) const {
    t->n_atoms = n_atoms;
    t->positions = positions.data();
    t->masses = masses.data();
    t->charges = charges.data();
    t->lj_sigma = lj_sigma.data();
    t->lj_epsilon = lj_epsilon.data();
    t->n_bonds = (int32_t)bonds.size();
    t->bonds = bonds.data();
    t->n_angles = (int32_t)angles.size();
    t->angles = angles.data();
    t->n_dihedrals = (int32_t)dihedrals.size();
    t->dihedrals = dihedrals.data();
    t->n_exceptions = (int32_t)exceptions.size();
    t->exceptions = exceptions.data();
    t->exclusion_offsets = exclusion_offsets.data();
    t->exclusions = exclusions.data();
    t->n_clusters = (int32_t)clusters.size();
    t->clusters = clusters.data();
  }
};

// Seeded poly-alanine-like chains (topology.cpp).  compact = 0: grown at
// `density` (atoms/Å^3) in their regions; compact = 1: grown sparse and then
// squeezed to `density` (sphere systems) or into the cube of edge box_edge.
// squeeze_stats (may be NULL, compact only): iterations, max contact overlap
// (Å), max wall violation (Å), closest pair more than three bonds apart (Å).
bool polyala_build(int n_chains, int n_res, uint64_t seed, double density, double box_edge,
                   HostTopology* T, std::string* err, int compact = 0, double* squeeze_stats = nullptr);

// Engine hooks for the job server (defined in engine.cu).  A job's topology is
// validated and lowered once on the submitting thread (prepare_system); the
// worker admits the lowered form into its batch (admit_prepared).  Errors are
// reported through prismq_last_error() of the calling thread.
void set_last_error(const std::string& msg);  // the message prismq_last_error() returns on this thread
struct PreparedSystem;
prismq_status prepare_system(const prismq_topology* t, const prismq_params* p, PreparedSystem** out);
void free_prepared(PreparedSystem* s);
int32_t prepared_atoms(const PreparedSystem* s);
prismq_status admit_prepared(prismq_batch* b, const PreparedSystem* s, int32_t* slot);
prismq_status batch_create_for_bytes(int64_t max_bytes, int32_t max_systems, prismq_batch** out,
                                     int64_t* atom_cap, int64_t* device_bytes);

}  // namespace pq

struct prismq_topology_buf {
  pq::HostTopology topo;
};
