"""Write tests/golden/prep_polyala_2x4.json: a PRISM-PREP topology document.

The system is the library's seeded poly-alanine builder (2 chains x 4
residues, seed 11, 80 atoms) written in the PrismPrepTopology schema
(crates/prism-nhs/src/input.rs:1027-1140) the way a PRISM-PREP / OpenMM run
writes it:
  * masses before repartitioning (N 14.01, C 12.01, O 16.00, H 1.008 amu),
    h_clusters carrying the matching inverse masses, and no hmr_applied key,
    so the load performs HMR x3;
  * bond and angle force constants in OPENMM_FULL_K_HALF_ENERGY form (twice
    the U = k (x - x0)^2 coefficient), declared by a sealed
    harmonic_parameter_contract;
  * strict exclusions (1-2, 1-3) and exact 1-4 nonbonded_exceptions with a
    sealed prismos_exact_nonbonded_exceptions_v2 contract.
Digests are sealed with oracle/prep_topology.py.  When a Prism-Q checkout is
given as argv[1], the harmonic contract is also checked with the reference's
own Python digest check (scripts/bind_biprism_harmonic_source.py:85-88).

Usage: python tests/golden/make_prep_json.py [PRISM_Q_CHECKOUT]
"""
from __future__ import annotations

import hashlib
import importlib
import importlib.util
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "prep_polyala_2x4.json"
N_CHAINS, N_RES, SEED = 2, 4, 11
NAMES = ("N", "H", "CA", "HA", "CB", "HB1", "HB2", "HB3", "C", "O")
ELEMENTS = ("N", "H", "C", "H", "C", "H", "H", "H", "C", "O")
MASS = {"N": 14.01, "C": 12.01, "O": 16.00, "H": 1.008}


def build_document() -> dict:
    sys.path.insert(0, str(ROOT))
    pq = importlib.import_module("prism-q_gb300")
    from oracle import prep_topology as prep

    t = pq.Topology.polyala(n_chains=N_CHAINS, n_residues=N_RES, seed=SEED)
    n = t.n_atoms
    f = lambda x: float(np.float32(x))  # noqa: E731  (the float32 value, written exactly)
    exc_pairs = {(int(e["i"]), int(e["j"])) for e in t.exceptions}
    strict = []
    for a in range(n):
        parts = [int(p) for p in t.exclusions[t.exclusion_offsets[a]:t.exclusion_offsets[a + 1]]]
        strict.append([p for p in parts if (min(a, p), max(a, p)) not in exc_pairs])
    mass0 = [MASS[ELEMENTS[a % 10]] for a in range(n)]
    clusters = []
    for c in t.clusters:
        nh = int(c["n_hydrogens"])
        clusters.append({"type": nh, "central_atom": int(c["central_atom"]),
                         "hydrogen_atoms": [int(h) for h in c["hydrogen_atoms"][:nh]],
                         "bond_lengths": [f(x) for x in c["bond_lengths"][:nh]], "n_hydrogens": nh,
                         "inv_mass_central": 1.0 / mass0[int(c["central_atom"])], "inv_mass_h": 1.0 / MASS["H"]})
    doc = {
        "source_pdb": "synthetic-polyala-2x4.pdb",
        "n_atoms": n,
        "n_residues": N_CHAINS * N_RES,
        "n_chains": N_CHAINS,
        "positions": [f(x) for x in t.positions.reshape(-1)],
        "elements": [ELEMENTS[a % 10] for a in range(n)],
        "atom_names": [NAMES[a % 10] for a in range(n)],
        "residue_names": ["ALA"] * n,
        "residue_ids": [a // 10 for a in range(n)],
        "chain_ids": ["AB"[a // (10 * N_RES)] for a in range(n)],
        "charges": [f(x) for x in t.charges],
        "masses": mass0,
        "ca_indices": [a for a in range(n) if a % 10 == 2],
        "bonds": [{"i": int(b["i"]), "j": int(b["j"]), "r0": f(b["r0"]), "k": 2.0 * f(b["k"])} for b in t.bonds],
        "angles": [{"i": int(a["i"]), "j": int(a["j"]), "k_idx": int(a["k"]), "theta0": f(a["theta0"]),
                    "force_k": 2.0 * f(a["force_k"])} for a in t.angles],
        "harmonic_parameter_contract": {
            "schema_kind": "prismos_harmonic_parameter_contract", "schema_version": 1,
            "source_provider": "synthetic-polyala:HarmonicBondForce+HarmonicAngleForce",
            "bond_convention": "OPENMM_FULL_K_HALF_ENERGY", "angle_convention": "OPENMM_FULL_K_HALF_ENERGY",
            "bond_coefficient_unit": "kcal/mol/angstrom^2", "angle_coefficient_unit": "kcal/mol/radian^2",
            "bond_equilibrium_unit": "angstrom", "angle_equilibrium_unit": "radian",
            "bond_uses_periodic_boundary_conditions": False, "angle_uses_periodic_boundary_conditions": False,
            "bond_count": 0, "angle_count": 0, "contract_sha256": ""},
        "dihedrals": [{"i": int(d["i"]), "j": int(d["j"]), "k_idx": int(d["k"]), "l": int(d["l"]),
                       "periodicity": int(d["periodicity"]), "phase": f(d["phase"]), "force_k": f(d["force_k"]),
                       "improper": False} for d in t.dihedrals],
        "lj_params": [{"sigma": f(s), "epsilon": f(e)} for s, e in zip(t.lj_sigma, t.lj_epsilon)],
        "exclusions": strict,
        "nonbonded_exceptions": [{"i": int(e["i"]), "j": int(e["j"]), "charge_product_e2": f(e["charge_product"]),
                                  "sigma_A": f(e["sigma"]), "epsilon_kcal_mol": f(e["epsilon"])}
                                 for e in t.exceptions],
        "nonbonded_exception_contract": {
            "schema_kind": "prismos_exact_nonbonded_exceptions_v2", "schema_version": 2,
            "semantics": "OPENMM_NONBONDEDFORCE_ABSOLUTE_EXCEPTION_PARAMETERS_V1",
            "dynamic_charge_scaling_semantics":
                "EXCITED_STATE_MULTIPLIES_GROUND_STATE_CHARGE_PRODUCT_BY_PER_ATOM_SCALE_PRODUCT_V1",
            "exact_scaled_pair_count": 0, "strict_exclusion_pair_count": 0, "total_openmm_exception_count": 0,
            "pair_digest_algorithm": "SHA256_PRISMOS_NBEX_ACTIVE_V1_LE_U64_U64_F64_F64_F64",
            "pair_digest_sha256": "",
            "strict_exclusion_digest_algorithm": "SHA256_PRISMOS_NBEX_STRICT_V1_LE_U64_U64",
            "strict_exclusion_digest_sha256": "", "source_prmtop_sha256": "",
            "hardcoded_uniform_scaling_allowed": False, "complete": True, "fallback_used": False},
        "generated_prmtop_sha256": hashlib.sha256(b"synthetic-polyala-2x4.prmtop").hexdigest(),
        "h_clusters": clusters,
    }
    return prep.seal(doc)


def check_with_reference(doc: dict, checkout: pathlib.Path) -> None:
    path = checkout / "scripts" / "bind_biprism_harmonic_source.py"
    spec = importlib.util.spec_from_file_location("ref_bind_harmonic", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.contract_hash(doc["harmonic_parameter_contract"])  # raises on a digest mismatch
    print("harmonic contract digest agrees with", path)


def main() -> None:
    doc = build_document()
    if len(sys.argv) > 1:
        check_with_reference(doc, pathlib.Path(sys.argv[1]))
    OUT.write_text(json.dumps(doc, separators=(",", ":")) + "\n")
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {doc['n_atoms']} atoms)")


if __name__ == "__main__":
    main()
