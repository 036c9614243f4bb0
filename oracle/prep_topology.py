"""CPU restatement of the PRISM-PREP topology load path (pure Python + numpy).

TEST INFRASTRUCTURE ONLY: the checker for the library's JSON ingest
(prismq_topology_from_prep_json).  Imported by tests/ and by the fixture
generator under tests/golden/; the product package never imports it.

Follows crates/prism-nhs/src/input.rs:
  python_canonical_json            :44-137   (== json.dumps(sort_keys=True,
                                              separators=(",", ":"), ensure_ascii=True),
                                              the form scripts/bind_biprism_harmonic_source.py:72-73 hashes)
  HarmonicParameterContract        :278-321  (fields, validate_for_topology)
  lower_harmonic_parameters        :467-520  (scale = source prefactor / 1.0, binary64 then float32)
  nonbonded_exception_digest_sha256 :1935-1949
  strict_exclusion_digest_sha256   :1952-1969
  validate                         :1996-2290
  validate_for_nonbonded_execution :1429-1450 (RequireExactV2)
  apply_hmr                        :2482-2560
Parity is pinned by the reference's own unit cases for these functions
(input.rs:2840-2960, :3245-3300, restated in tests/test_prep_json.py) and by the
reference's Python contract check (bind_biprism_harmonic_source.py:85-88),
which the fixture generator runs on the committed fixture.
"""
from __future__ import annotations

import hashlib
import json
import math
import struct

import numpy as np

BOND_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("r0", "<f4"), ("k", "<f4")])
ANGLE_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("theta0", "<f4"), ("force_k", "<f4")])
DIH_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("l", "<i4"), ("periodicity", "<i4"),
                   ("phase", "<f4"), ("force_k", "<f4")])
EXC_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("charge_product", "<f4"), ("sigma", "<f4"), ("epsilon", "<f4")])
CLUSTER_DT = np.dtype([("central_atom", "<i4"), ("hydrogen_atoms", "<i4", (3,)), ("bond_lengths", "<f4", (3,)),
                       ("n_hydrogens", "<i4"), ("inv_mass_central", "<f4"), ("inv_mass_h", "<f4")])

PREFACTOR = {"OPENMM_FULL_K_HALF_ENERGY": 0.5, "AMBER_NO_HALF_ENERGY": 1.0}  # input.rs:264-270
HARMONIC_FIELDS = ("schema_kind", "schema_version", "source_provider", "bond_convention", "angle_convention",
                   "bond_coefficient_unit", "angle_coefficient_unit", "bond_equilibrium_unit",
                   "angle_equilibrium_unit", "bond_uses_periodic_boundary_conditions",
                   "angle_uses_periodic_boundary_conditions", "bond_count", "angle_count", "contract_sha256")


class Refused(ValueError):
    """The reference would refuse this topology; the message names the rule."""


def _require(cond, msg):
    if not cond:
        raise Refused(msg)


def canonical(value) -> bytes:
    return json.dumps(value, sort_keys=True, separators=(",", ":"), ensure_ascii=True).encode()


def harmonic_contract_digest(contract: dict) -> str:
    body = {k: v for k, v in contract.items() if k != "contract_sha256"}
    return hashlib.sha256(canonical(body)).hexdigest()


def exception_digest(exceptions) -> str:
    rows = sorted(exceptions, key=lambda r: (r["i"], r["j"]))
    h = hashlib.sha256(b"PRISMOS_NBEX_ACTIVE_V1\0" + struct.pack("<Q", len(rows)))
    for r in rows:
        h.update(struct.pack("<QQddd", r["i"], r["j"], r["charge_product_e2"], r["sigma_A"], r["epsilon_kcal_mol"]))
    return h.hexdigest()


def strict_pairs(exclusions) -> list:
    return sorted({(min(a, p), max(a, p)) for a, parts in enumerate(exclusions) for p in parts})


def strict_digest(exclusions) -> str:
    pairs = strict_pairs(exclusions)
    h = hashlib.sha256(b"PRISMOS_NBEX_STRICT_V1\0" + struct.pack("<Q", len(pairs)))
    for i, j in pairs:
        h.update(struct.pack("<QQ", i, j))
    return h.hexdigest()


def _is_uint(v) -> bool:
    return type(v) is int and v >= 0


def _f32(x) -> np.float32:
    return np.float32(float(x))


def validate(doc: dict) -> None:
    """PrismPrepTopology::validate (input.rs:1996-2290), the path's fields."""
    n = doc["n_atoms"]
    _require(_is_uint(n) and n > 0, "n_atoms must be a positive integer")
    h = doc.get("harmonic_parameter_contract")
    if h is not None:
        _require(set(h) <= set(HARMONIC_FIELDS), "harmonic_parameter_contract: unknown field")
        _require(set(h) == set(HARMONIC_FIELDS), "harmonic_parameter_contract: missing field")
        _require(h["bond_convention"] in PREFACTOR and h["angle_convention"] in PREFACTOR,
                 "unknown harmonic energy convention")
        ok = (h["schema_kind"] == "prismos_harmonic_parameter_contract" and h["schema_version"] == 1
              and h["source_provider"].strip() != ""
              and h["bond_coefficient_unit"] == "kcal/mol/angstrom^2"
              and h["angle_coefficient_unit"] == "kcal/mol/radian^2"
              and h["bond_equilibrium_unit"] == "angstrom" and h["angle_equilibrium_unit"] == "radian"
              and h["bond_uses_periodic_boundary_conditions"] is False
              and h["angle_uses_periodic_boundary_conditions"] is False
              and h["bond_count"] == len(doc["bonds"]) and h["angle_count"] == len(doc["angles"]))
        _require(ok, "harmonic source contract has unsupported schema, units, provider or term counts")
        _require(h["contract_sha256"] == harmonic_contract_digest(h),
                 "harmonic source contract canonical digest mismatch")
    _require(len(doc["positions"]) == 3 * n, "positions length != expected")
    for key in ("elements", "atom_names", "residue_names", "residue_ids", "chain_ids", "charges", "masses",
                "lj_params", "exclusions"):
        _require(len(doc[key]) == n, f"{key} length != expected")
    _require(max(doc["residue_ids"], default=0) < doc["n_residues"], "max residue_id >= n_residues")
    _require(all(math.isfinite(_f32(v)) for v in doc["positions"]), "position value is non-finite")
    _require(all(math.isfinite(_f32(v)) for v in doc["charges"]), "charge value is non-finite")
    _require(all(math.isfinite(_f32(v)) and _f32(v) > 0 for v in doc["masses"]),
             "mass value must be finite and positive")
    for lj in doc["lj_params"]:
        s, e = lj["sigma"], lj["epsilon"]
        _require(math.isfinite(s) and math.isfinite(e) and s >= 0 and e >= 0, "invalid LJ parameters")
    ca = doc["ca_indices"]
    _require(all(_is_uint(i) and i < n for i in ca) and len(set(ca)) == len(ca),
             "invalid or duplicate CA atom index")
    for b in doc["bonds"]:
        _require(b["i"] < n and b["j"] < n and b["i"] != b["j"] and math.isfinite(b["r0"]) and math.isfinite(b["k"])
                 and b["r0"] > 0 and b["k"] >= 0, "invalid bond term")
    for a in doc["angles"]:
        i, j, k = a["i"], a["j"], a["k_idx"]
        _require(i < n and j < n and k < n and len({i, j, k}) == 3 and math.isfinite(a["theta0"])
                 and math.isfinite(a["force_k"]) and 0 < a["theta0"] <= math.pi and a["force_k"] >= 0,
                 "invalid angle term")
    for d in doc["dihedrals"]:
        _require(all(d[x] < n for x in ("i", "j", "k_idx", "l")) and d.get("periodicity", 0) > 0
                 and math.isfinite(d.get("phase", 0.0)) and math.isfinite(d.get("force_k", 0.0)),
                 "invalid dihedral term")
    excl = doc["exclusions"]
    for a, parts in enumerate(excl):
        _require(all(_is_uint(p) and p < n and p != a for p in parts) and len(set(parts)) == len(parts),
                 "invalid, self, or duplicate strict exclusion")
        _require(all(a in excl[p] for p in parts), "asymmetric strict exclusion")
    strict = set(strict_pairs(excl))
    seen = set()
    exc = doc.get("nonbonded_exceptions", [])
    for e in exc:
        i, j = e["i"], e["j"]
        _require(i < n and j < n, "nonbonded exception index out of range")
        _require(i < j, "nonbonded exception pair must be canonical i < j")
        vals = (e["charge_product_e2"], e["sigma_A"], e["epsilon_kcal_mol"])
        _require(all(math.isfinite(v) for v in vals) and vals[1] >= 0 and vals[2] >= 0,
                 "invalid nonbonded exception parameters")
        for v in vals:
            nv = _f32(v)
            _require(math.isfinite(nv) and not (v != 0 and nv == 0) and not (v == 0 and math.copysign(1, v) < 0),
                     "nonbonded exception is not safely representable as f32")
            _require(abs(float(nv) - v) <= max(1e-12, abs(v) * 1e-6), "nonbonded exception f32 conversion error")
        _require((i, j) not in seen, "duplicate nonbonded exception pair")
        seen.add((i, j))
        _require((i, j) not in strict, "nonbonded exception overlaps strict exclusion")
    c = doc.get("nonbonded_exception_contract")
    _require(not (not exc and c is not None), "nonbonded exception contract is present but the exact pair vector is empty")
    _require(not (exc and c is None), "exact nonbonded exceptions require a versioned completeness/digest contract")
    if c is not None:
        _require(c["schema_kind"] == "prismos_exact_nonbonded_exceptions_v2" and c["schema_version"] == 2,
                 "unsupported nonbonded exception contract")
        _require(c["semantics"] == "OPENMM_NONBONDEDFORCE_ABSOLUTE_EXCEPTION_PARAMETERS_V1"
                 and c["dynamic_charge_scaling_semantics"]
                 == "EXCITED_STATE_MULTIPLIES_GROUND_STATE_CHARGE_PRODUCT_BY_PER_ATOM_SCALE_PRODUCT_V1",
                 "unsupported exact nonbonded exception semantics")
        _require(c["pair_digest_algorithm"] == "SHA256_PRISMOS_NBEX_ACTIVE_V1_LE_U64_U64_F64_F64_F64"
                 and c["strict_exclusion_digest_algorithm"] == "SHA256_PRISMOS_NBEX_STRICT_V1_LE_U64_U64",
                 "unsupported nonbonded exception digest algorithms")
        _require(c["complete"] and not c["fallback_used"] and not c["hardcoded_uniform_scaling_allowed"],
                 "exact nonbonded exception contract is incomplete or records fallback")
        _require(c["exact_scaled_pair_count"] == len(exc), "nonbonded exception count mismatch")
        _require(c["strict_exclusion_pair_count"] == len(strict), "strict exclusion count mismatch")
        _require(c["total_openmm_exception_count"] == len(exc) + len(strict), "OpenMM exception completeness mismatch")
        _require(c["pair_digest_sha256"] == exception_digest(exc), "nonbonded exception digest mismatch")
        _require(c["strict_exclusion_digest_sha256"] == strict_digest(excl), "strict exclusion digest mismatch")
        prm = doc.get("generated_prmtop_sha256")
        _require(prm is not None, "exact nonbonded exceptions require generated_prmtop_sha256 provenance")
        _require(c["source_prmtop_sha256"] == prm and len(prm) == 64
                 and all(ch in "0123456789abcdefABCDEF" for ch in prm),
                 "exact exception source prmtop hash is absent, malformed, or mismatched")


def lower(doc: dict, apply_hmr: bool = True, hmr_factor: float = 3.0, require_harmonic_contract: bool = True,
          require_exceptions: bool = True) -> dict:
    """The topology the engine receives, as numpy arrays in the C ABI's layouts, plus a report."""
    validate(doc)
    exc = doc.get("nonbonded_exceptions", [])
    if require_exceptions:  # RequireExactV2 (input.rs:1438-1447)
        _require(exc and doc.get("nonbonded_exception_contract") is not None,
                 "production nonbonded execution requires exact OpenMM exception parameters and a complete V2 contract")
    h = doc.get("harmonic_parameter_contract")
    _require(h is not None or not require_harmonic_contract,
             "harmonic source convention is absent: refusing production lowering")
    for b in doc["bonds"]:
        _require(math.isfinite(_f32(b["r0"])) and _f32(b["r0"]) > 0, "harmonic equilibrium coordinate")
    for a in doc["angles"]:
        _require(math.isfinite(_f32(a["theta0"])) and _f32(a["theta0"]) > 0, "harmonic equilibrium coordinate")
    bond_scale = PREFACTOR[h["bond_convention"]] / 1.0 if h else 1.0
    angle_scale = PREFACTOR[h["angle_convention"]] / 1.0 if h else 1.0

    def cast(raw, scale):
        mapped = raw * scale
        dev = _f32(mapped)
        _require(math.isfinite(raw) and raw >= 0 and math.isfinite(mapped) and math.isfinite(dev)
                 and not (raw > 0 and dev == 0), "coefficient is invalid or not representable")
        return dev

    n = doc["n_atoms"]
    out = {
        "positions": np.array(doc["positions"], dtype=np.float64).astype(np.float32).reshape(n, 3),
        "masses": np.array(doc["masses"], dtype=np.float64).astype(np.float32),
        "charges": np.array(doc["charges"], dtype=np.float64).astype(np.float32),
        "lj_sigma": np.array([lj["sigma"] for lj in doc["lj_params"]], dtype=np.float64).astype(np.float32),
        "lj_epsilon": np.array([lj["epsilon"] for lj in doc["lj_params"]], dtype=np.float64).astype(np.float32),
    }
    out["bonds"] = np.array([(b["i"], b["j"], _f32(b["r0"]), cast(b["k"], bond_scale)) for b in doc["bonds"]],
                            dtype=BOND_DT)
    out["angles"] = np.array([(a["i"], a["j"], a["k_idx"], _f32(a["theta0"]), cast(a["force_k"], angle_scale))
                              for a in doc["angles"]], dtype=ANGLE_DT)
    out["dihedrals"] = np.array([(d["i"], d["j"], d["k_idx"], d["l"], d.get("periodicity", 0),
                                  _f32(d.get("phase", 0.0)), _f32(d.get("force_k", 0.0))) for d in doc["dihedrals"]],
                                dtype=DIH_DT)
    out["exceptions"] = np.array([(e["i"], e["j"], _f32(e["charge_product_e2"]), _f32(e["sigma_A"]),
                                   _f32(e["epsilon_kcal_mol"])) for e in exc], dtype=EXC_DT)
    offs = [0]
    flat = []
    for parts in doc["exclusions"]:
        flat.extend(parts)
        offs.append(len(flat))
    out["exclusion_offsets"] = np.array(offs, dtype=np.int32)
    out["exclusions"] = np.array(flat, dtype=np.int32)
    # hydrogen mass repartitioning (input.rs:2482-2560), binary64 on the inverse masses
    clusters = [dict(c) for c in doc.get("h_clusters", [])]
    report = {"hmr_performed": 0, "n_repartitioned": 0, "n_skipped": 0, "exact_exceptions": len(exc),
              "bond_scale": bond_scale, "angle_scale": angle_scale, "total_mass_before": 0.0,
              "total_mass_after": 0.0}
    if apply_hmr and doc.get("hmr_applied") is not True:
        report["hmr_performed"] = 1
        for c in clusters:
            m_h = 1.0 / c["inv_mass_h"]
            m_c = 1.0 / c["inv_mass_central"]
            nh = float(c["n_hydrogens"])
            report["total_mass_before"] += m_c + nh * m_h
            m_h_new = m_h * hmr_factor
            dm = m_h_new - m_h
            m_c_new = m_c - nh * dm
            if m_c_new < 1.0:
                report["total_mass_after"] += m_c + nh * m_h
                report["n_skipped"] += 1
                continue
            c["inv_mass_h"] = 1.0 / m_h_new
            c["inv_mass_central"] = 1.0 / m_c_new
            report["n_repartitioned"] += 1
            report["total_mass_after"] += m_c_new + nh * m_h_new
            out["masses"][c["central_atom"]] = np.float32(m_c_new)
            for hh in c["hydrogen_atoms"]:
                if hh >= 0:
                    out["masses"][hh] = np.float32(m_h_new)
    rows = []
    for c in clusters:
        hyd = list(c["hydrogen_atoms"]) + [-1] * (3 - len(c["hydrogen_atoms"]))
        lens = list(c["bond_lengths"]) + [0.0] * (3 - len(c["bond_lengths"]))
        rows.append((c["central_atom"], hyd, [_f32(x) for x in lens], c["n_hydrogens"],
                     _f32(c["inv_mass_central"]), _f32(c["inv_mass_h"])))
    out["clusters"] = np.array(rows, dtype=CLUSTER_DT)
    out["report"] = report
    return out


def seal(doc: dict) -> dict:
    """Fill the contract digests of a topology document in place (fixture writing)."""
    h = doc.get("harmonic_parameter_contract")
    if h is not None:
        h["bond_count"], h["angle_count"] = len(doc["bonds"]), len(doc["angles"])
        h["contract_sha256"] = harmonic_contract_digest(h)
    c = doc.get("nonbonded_exception_contract")
    if c is not None:
        exc = doc.get("nonbonded_exceptions", [])
        strict = strict_pairs(doc["exclusions"])
        c["exact_scaled_pair_count"] = len(exc)
        c["strict_exclusion_pair_count"] = len(strict)
        c["total_openmm_exception_count"] = len(exc) + len(strict)
        c["pair_digest_sha256"] = exception_digest(exc)
        c["strict_exclusion_digest_sha256"] = strict_digest(doc["exclusions"])
        c["source_prmtop_sha256"] = doc.get("generated_prmtop_sha256")
    return doc
