// TEST INFRASTRUCTURE ONLY.  The library's synthetic-system generator
// (prism-q_gb300/csrc/topology.cpp, host code) built into the oracle's own
// shared object, so that the CPU legs of the benchmark build their inputs
// without loading the product library.  Loaded by oracle/oracle.py.
#include <cstring>
#include <string>

#include "../prism-q_gb300/csrc/pq_host.h"

extern "C" {

// A new topology, or NULL with the reason in err (err_cap bytes).
void* orcgen_polyala(int n_chains, int n_res, unsigned long long seed, double density, double box_edge, int compact,
                     double* stats, char* err, int err_cap) {
  auto* T = new pq::HostTopology();
  std::string msg;
  if (!pq::polyala_build(n_chains, n_res, seed, density, box_edge, T, &msg, compact, stats)) {
    if (err && err_cap > 0) {
      std::strncpy(err, msg.c_str(), (size_t)err_cap - 1);
      err[err_cap - 1] = 0;
    }
    delete T;
    return nullptr;
  }
  return T;
}

void orcgen_view(void* h, prismq_topology* out) { static_cast<pq::HostTopology*>(h)->view(out); }

void orcgen_free(void* h) { delete static_cast<pq::HostTopology*>(h); }
}
