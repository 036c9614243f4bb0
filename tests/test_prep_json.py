"""PRISM-PREP topology JSON ingest (prismq_topology_from_prep_json) against the
oracle restatement of the reference's load path (oracle/prep_topology.py).

Bar: bit-exact (the lowering is integer / IEEE cast work) for every array the
engine receives, agreement on which documents are refused, and on the GPU,
forces of the ingested system bit-identical to the builder's and within
1e-5 relative RMS of the FP64 oracle.

The small hand-built documents restate the reference's own unit cases for this
path (crates/prism-nhs/src/input.rs:2840-2960 minimal / exact topologies,
:3245-3300 HMR authority and JSON value bits, and the v2 contract mutation
cases that follow them).
"""
from __future__ import annotations

import copy
import ctypes
import hashlib
import json
import struct

import numpy as np
import pytest

from conftest import ROOT, rel_rms
from oracle import prep_topology as prep

FIXTURE = ROOT / "tests" / "golden" / "prep_polyala_2x4.json"
ARRAYS = ("positions", "masses", "charges", "lj_sigma", "lj_epsilon", "bonds", "angles", "dihedrals", "exceptions",
          "exclusion_offsets", "exclusions", "clusters")


@pytest.fixture(scope="module")
def doc():
    return json.loads(FIXTURE.read_text())


def _ingest(pq, d, **kw):
    rep = {}
    t = pq.Topology.from_prep_json(json.dumps(d), report=rep, **kw)
    return t, rep


def _same(pq, d, **kw):
    """Both sides load `d` and agree bit for bit, or both refuse it."""
    try:
        want = prep.lower(d, **kw)
    except prep.Refused as e:
        with pytest.raises(pq.PrismQError) as got:
            _ingest(pq, d, **kw)
        assert got.value.status == 1
        return None, str(e), str(got.value)
    t, rep = _ingest(pq, d, **kw)
    for k in ARRAYS:
        a, b = getattr(t, k), want[k]
        assert a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes(), k
    assert rep == want["report"]
    return t, None, None


def _minimal():
    """The reference's 5-atom minimal topology (input.rs:2840-2909)."""
    return {
        "source_pdb": "test.pdb", "n_atoms": 5, "n_residues": 2, "n_chains": 1,
        "positions": [0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 2.0, 0.0, 0.0, 3.0, 0.0, 0.0, 4.0, 0.0, 0.0],
        "elements": ["C", "N", "O", "C", "C"], "atom_names": ["CA", "N", "O", "CB", "CG"],
        "residue_names": ["ALA", "ALA", "ALA", "PHE", "PHE"], "residue_ids": [0, 0, 0, 1, 1],
        "chain_ids": ["A"] * 5, "charges": [0.0] * 5, "masses": [12.0, 14.0, 16.0, 12.0, 12.0],
        "ca_indices": [0], "bonds": [], "angles": [], "dihedrals": [],
        "lj_params": [{"sigma": 1.5, "epsilon": 0.1}] * 5, "exclusions": [[] for _ in range(5)],
        "nonbonded_exceptions": [], "nonbonded_exception_contract": None, "generated_prmtop_sha256": None,
        "h_clusters": [], "hmr_applied": False,
    }


def _exact():
    """The reference's exact-exception topology (input.rs:2911-2943)."""
    d = _minimal()
    d["exclusions"][0].append(1)
    d["exclusions"][1].append(0)
    d["nonbonded_exceptions"] = [{"i": 0, "j": 3, "charge_product_e2": -0.125, "sigma_A": 3.5,
                                  "epsilon_kcal_mol": 0.025}]
    d["generated_prmtop_sha256"] = "a" * 64
    d["nonbonded_exception_contract"] = {
        "schema_kind": "prismos_exact_nonbonded_exceptions_v2", "schema_version": 2,
        "semantics": "OPENMM_NONBONDEDFORCE_ABSOLUTE_EXCEPTION_PARAMETERS_V1",
        "dynamic_charge_scaling_semantics":
            "EXCITED_STATE_MULTIPLIES_GROUND_STATE_CHARGE_PRODUCT_BY_PER_ATOM_SCALE_PRODUCT_V1",
        "exact_scaled_pair_count": 1, "strict_exclusion_pair_count": 1, "total_openmm_exception_count": 2,
        "pair_digest_algorithm": "SHA256_PRISMOS_NBEX_ACTIVE_V1_LE_U64_U64_F64_F64_F64",
        "pair_digest_sha256": prep.exception_digest(d["nonbonded_exceptions"]),
        "strict_exclusion_digest_algorithm": "SHA256_PRISMOS_NBEX_STRICT_V1_LE_U64_U64",
        "strict_exclusion_digest_sha256": prep.strict_digest(d["exclusions"]),
        "source_prmtop_sha256": "a" * 64, "hardcoded_uniform_scaling_allowed": False, "complete": True,
        "fallback_used": False}
    return d


NOCONTRACT = {"require_harmonic_contract": False}


# ---------------------------------------------------------------- fixture
def test_fixture_bit_exact_with_oracle(pq, doc):
    t, _, _ = _same(pq, doc)
    assert t.n_atoms == 80


def test_fixture_lowers_to_the_builder_topology(pq, doc):
    """OPENMM full-k halved to U = k (x - x0)^2 and HMR x3 reproduce the
    builder's own arrays exactly; exception pairs stay out of the strict list."""
    t, rep = _ingest(pq, doc)
    b = pq.Topology.polyala(2, 4, seed=11)
    for k in ("positions", "masses", "charges", "lj_sigma", "lj_epsilon", "bonds", "angles", "dihedrals",
              "exceptions", "clusters"):
        assert getattr(t, k).tobytes() == getattr(b, k).tobytes(), k
    assert rep["hmr_performed"] == 1 and rep["n_repartitioned"] == len(b.clusters) and rep["n_skipped"] == 0
    assert rep["bond_scale"] == 0.5 and rep["angle_scale"] == 0.5
    assert abs(rep["total_mass_after"] - rep["total_mass_before"]) < 1e-9
    strict = {(a, int(p)) for a in range(t.n_atoms) for p in t.exclusions[t.exclusion_offsets[a]:t.exclusion_offsets[a + 1]]}
    assert not any((int(e["i"]), int(e["j"])) in strict for e in t.exceptions)


def test_fixture_file_and_text_paths_agree(pq, doc):
    a = pq.Topology.from_prep_json(str(FIXTURE))
    b = pq.Topology.from_prep_json(FIXTURE.read_bytes())
    for k in ARRAYS:
        assert getattr(a, k).tobytes() == getattr(b, k).tobytes()
    with pytest.raises(pq.PrismQError) as e:
        pq.Topology.from_prep_json(str(FIXTURE) + ".missing")
    assert e.value.status == 11


def test_fixture_contract_digests(doc):
    h = doc["harmonic_parameter_contract"]
    assert h["contract_sha256"] == prep.harmonic_contract_digest(h)
    c = doc["nonbonded_exception_contract"]
    assert c["pair_digest_sha256"] == prep.exception_digest(doc["nonbonded_exceptions"])
    assert c["strict_exclusion_digest_sha256"] == prep.strict_digest(doc["exclusions"])


def test_amber_convention_keeps_k(pq, doc):
    d = copy.deepcopy(doc)
    d["harmonic_parameter_contract"]["bond_convention"] = "AMBER_NO_HALF_ENERGY"
    prep.seal(d)
    t, _, _ = _same(pq, d)
    assert np.array_equal(t.bonds["k"], np.array([b["k"] for b in d["bonds"]], np.float32))
    assert np.array_equal(t.angles["force_k"], np.array([a["force_k"] * 0.5 for a in d["angles"]], np.float32))


@pytest.mark.parametrize("factor", [2.0, 3.0, 4.0])
def test_hmr_factor(pq, doc, factor):
    t, _, _ = _same(pq, doc, hmr_factor=factor)
    h = [int(hh) for c in t.clusters for hh in c["hydrogen_atoms"] if hh >= 0]
    assert np.all(t.masses[h] == np.float32(1.0 / (1.0 / 1.008) * factor))


def test_hmr_recorded_true_preserves_masses(pq, doc):
    d = copy.deepcopy(doc)
    d["hmr_applied"] = True
    t, _, _ = _same(pq, d)
    assert np.array_equal(t.masses, np.array(d["masses"], np.float32))
    _, rep = _ingest(pq, d)
    assert rep["hmr_performed"] == 0


def test_hmr_disabled_by_option(pq, doc):
    t, _, _ = _same(pq, doc, apply_hmr=False)
    assert np.array_equal(t.masses, np.array(doc["masses"], np.float32))


# ---------------------------------------------------------------- the reference's unit cases
def test_minimal_topology_refused_by_production_policy(pq):
    _, want, got = _same(pq, _minimal(), **NOCONTRACT)
    assert "production nonbonded execution requires exact" in want
    assert "production nonbonded execution requires exact" in got


def test_minimal_topology_loads_under_nonproduction_policy(pq):
    t, _, _ = _same(pq, _minimal(), require_exceptions=False, **NOCONTRACT)
    assert t.n_atoms == 5 and len(t.exceptions) == 0


def test_harmonic_contract_required_by_default(pq):
    _, want, got = _same(pq, _exact())
    assert "harmonic source convention is absent" in want and "harmonic source convention is absent" in got


def test_exact_topology_accepted(pq):
    t, _, _ = _same(pq, _exact(), **NOCONTRACT)
    assert t.exceptions.tolist() == [(0, 3, -0.125, 3.5, np.float32(0.025))]
    assert t.exclusions.tolist() == [1, 0]


def test_exception_json_value_bits():
    """serde's binary64 parse of the reference's exception row (input.rs:3284-3296);
    the library reads numbers with the correctly rounded strtod, as Python does."""
    row = json.loads('{"i":1,"j":14,"charge_product_e2":0.09932701675511141,'
                     '"sigma_A":2.234373985145219,"epsilon_kcal_mol":0.018372533883399215}')
    bits = [struct.unpack("<Q", struct.pack("<d", row[k]))[0]
            for k in ("charge_product_e2", "sigma_A", "epsilon_kcal_mol")]
    assert bits == [0x3FB96D7ED0928BEC, 0x4001DFFF77C9DAF1, 0x3F92D03FE0B20621]


def test_exception_json_value_bits_reach_the_digest(pq):
    d = _exact()
    d["n_atoms"] = 15
    for key in ("elements", "atom_names", "residue_names", "chain_ids"):
        d[key] = d[key] + [d[key][-1]] * 10
    d["residue_ids"] = d["residue_ids"] + [1] * 10
    d["charges"] = [0.0] * 15
    d["masses"] = d["masses"] + [12.0] * 10
    d["positions"] = [float(x) for a in range(15) for x in (a, 0.0, 0.0)]
    d["lj_params"] = [{"sigma": 1.5, "epsilon": 0.1}] * 15
    d["exclusions"] = d["exclusions"] + [[] for _ in range(10)]
    d["nonbonded_exceptions"] = [{"i": 1, "j": 14, "charge_product_e2": 0.09932701675511141,
                                  "sigma_A": 2.234373985145219, "epsilon_kcal_mol": 0.018372533883399215}]
    prep.seal(d)
    t, _, _ = _same(pq, d, **NOCONTRACT)
    assert t.exceptions["charge_product"][0] == np.float32(0.09932701675511141)
    # one binary64 ulp off in the text changes the pair digest: the library refuses
    text = json.dumps(d).replace("0.09932701675511141", "0.09932701675511142")
    with pytest.raises(pq.PrismQError) as e:
        pq.Topology.from_prep_json(text, **NOCONTRACT)
    assert "digest mismatch" in str(e.value)


def test_hmr_respects_serialized_preapplied_authority(pq):
    d = _minimal()
    d["masses"][0], d["masses"][1] = 9.0, 3.0
    d["h_clusters"] = [{"type": 1, "central_atom": 0, "hydrogen_atoms": [1], "bond_lengths": [1.0],
                        "n_hydrogens": 1, "inv_mass_central": 1.0 / 9.0, "inv_mass_h": 1.0 / 3.0}]
    d["hmr_applied"] = True
    kw = dict(require_exceptions=False, **NOCONTRACT)
    t, _, _ = _same(pq, d, **kw)
    assert t.masses[:2].tolist() == [9.0, 3.0]
    assert t.clusters[0]["inv_mass_central"] == np.float32(1.0 / 9.0)
    for flag in (False, None):  # an unverified record repartitions
        d2 = copy.deepcopy(d)
        if flag is None:
            del d2["hmr_applied"]
        else:
            d2["hmr_applied"] = flag
        t, _, _ = _same(pq, d2, **kw)
        assert t.masses[:2].tolist() == [3.0, 9.0]  # m_h 3 -> 9, central 9 -> 9 - 6


def test_hmr_skips_cluster_whose_central_atom_would_drop_below_one_amu(pq):
    d = _minimal()
    d["masses"][0], d["masses"][1] = 2.0, 1.0
    d["h_clusters"] = [{"type": 1, "central_atom": 0, "hydrogen_atoms": [1], "bond_lengths": [1.0],
                        "n_hydrogens": 1, "inv_mass_central": 0.5, "inv_mass_h": 1.0}]
    t, _, _ = _same(pq, d, require_exceptions=False, **NOCONTRACT)
    assert t.masses[:2].tolist() == [2.0, 1.0]
    _, rep = _ingest(pq, d, require_exceptions=False, **NOCONTRACT)
    assert rep["n_skipped"] == 1 and rep["n_repartitioned"] == 0


# ---------------------------------------------------------------- refusals
def _mutations():
    def m(name, fn, **kw):
        return pytest.param(fn, kw, id=name)

    def set_path(path, value, reseal=False):
        def f(d):
            obj = d
            for k in path[:-1]:
                obj = obj[k]
            obj[path[-1]] = value
            if reseal:
                prep.seal(d)
        return f

    def exc_mut(d):
        d["nonbonded_exceptions"][0]["charge_product_e2"] += 0.5

    def strict_add(d):  # a new strict pair (symmetric) without resealing
        d["exclusions"][2].append(4)
        d["exclusions"][4].append(2)

    def asym(d):
        d["exclusions"][2].append(4)

    def dup(d):
        d["exclusions"][0].append(1)

    def self_excl(d):
        d["exclusions"][2].append(2)

    def oob_excl(d):
        d["exclusions"][2].append(5)

    def overlap(d):
        d["exclusions"][0].append(3)
        d["exclusions"][3].append(0)
        prep.seal(d)

    def noncanonical(d):
        e = d["nonbonded_exceptions"][0]
        e["i"], e["j"] = e["j"], e["i"]
        prep.seal(d)

    def duplicate_exc(d):
        d["nonbonded_exceptions"].append(dict(d["nonbonded_exceptions"][0]))
        prep.seal(d)

    def f32_lossy(d):
        d["nonbonded_exceptions"][0]["epsilon_kcal_mol"] = 1.0e-50  # underflows float32 to 0
        prep.seal(d)

    def negative_zero(d):
        d["nonbonded_exceptions"][0]["charge_product_e2"] = -0.0
        prep.seal(d)

    def contract_without_pairs(d):
        d["nonbonded_exceptions"] = []

    def no_contract(d):
        d["nonbonded_exception_contract"] = None

    def bad_bond(d):
        d["bonds"] = [{"i": 0, "j": 0, "r0": 1.0, "k": 1.0}]

    def neg_k(d):
        d["bonds"] = [{"i": 0, "j": 1, "r0": 1.0, "k": -1.0}]

    def bad_angle(d):
        d["angles"] = [{"i": 0, "j": 1, "k_idx": 2, "theta0": 3.5, "force_k": 1.0}]

    def zero_periodicity(d):
        d["dihedrals"] = [{"i": 0, "j": 1, "k_idx": 2, "l": 3, "phase": 0.0, "force_k": 1.0}]

    def short_masses(d):
        d["masses"] = d["masses"][:4]

    def zero_mass(d):
        d["masses"][2] = 0.0

    def bad_lj(d):
        d["lj_params"] = [{"sigma": 1.5, "epsilon": 0.1}] * 4 + [{"sigma": -1.0, "epsilon": 0.1}]

    def bad_resid(d):
        d["residue_ids"][4] = 2

    def dup_ca(d):
        d["ca_indices"] = [0, 0]

    def float_index(d):
        d["ca_indices"] = [1.0]

    def prmtop_mismatch(d):
        d["generated_prmtop_sha256"] = "b" * 64

    def prmtop_absent(d):
        d["generated_prmtop_sha256"] = None

    def missing_key(d):
        del d["chain_ids"]

    return [
        m("active_pair_mutation", exc_mut),
        m("strict_set_mutation", strict_add),
        m("asymmetric_exclusion", asym),
        m("duplicate_exclusion", dup),
        m("self_exclusion", self_excl),
        m("out_of_range_exclusion", oob_excl),
        m("exception_overlaps_strict", overlap),
        m("exception_not_canonical", noncanonical),
        m("duplicate_exception", duplicate_exc),
        m("exception_not_f32_exact", f32_lossy),
        m("exception_negative_zero", negative_zero),
        m("contract_without_pairs", contract_without_pairs, require_exceptions=False),
        m("pairs_without_contract", no_contract, require_exceptions=False),
        m("contract_schema", set_path(["nonbonded_exception_contract", "schema_version"], 1)),
        m("contract_incomplete", set_path(["nonbonded_exception_contract", "complete"], False)),
        m("contract_fallback", set_path(["nonbonded_exception_contract", "fallback_used"], True)),
        m("contract_count", set_path(["nonbonded_exception_contract", "total_openmm_exception_count"], 3)),
        m("prmtop_mismatch", prmtop_mismatch),
        m("prmtop_absent", prmtop_absent),
        m("bond_self", bad_bond),
        m("bond_negative_k", neg_k),
        m("angle_above_pi", bad_angle),
        m("dihedral_periodicity_default_zero", zero_periodicity),
        m("length_mismatch", short_masses),
        m("zero_mass", zero_mass),
        m("negative_sigma", bad_lj),
        m("residue_id_range", bad_resid),
        m("duplicate_ca", dup_ca),
        m("index_written_as_float", float_index),
        m("missing_required_key", missing_key),
    ]


@pytest.mark.parametrize("mutate,kw", _mutations())
def test_mutation_refused_by_both(pq, mutate, kw):
    d = _exact()
    mutate(d)
    opts = dict(NOCONTRACT)
    opts.update(kw)
    if mutate.__name__ in ("float_index", "missing_key"):
        with pytest.raises(pq.PrismQError) as e:  # serde refuses these before validation
            _ingest(pq, d, **opts)
        assert e.value.status == 1
        return
    t, want, got = _same(pq, d, **opts)
    assert t is None, "both sides should refuse"


def _harmonic_doc():
    d = _exact()
    d["bonds"] = [{"i": 0, "j": 1, "r0": 1.5, "k": 600.0}, {"i": 3, "j": 4, "r0": 1.4, "k": 1e-44}]
    d["angles"] = [{"i": 0, "j": 1, "k_idx": 2, "theta0": 1.9, "force_k": 100.0}]
    d["exclusions"] = [[1, 2], [0, 2], [0, 1], [4], [3]]
    d["harmonic_parameter_contract"] = {
        "schema_kind": "prismos_harmonic_parameter_contract", "schema_version": 1,
        "source_provider": "OpenMM/8.1.1:HarmonicBondForce+HarmonicAngleForce",
        "bond_convention": "OPENMM_FULL_K_HALF_ENERGY", "angle_convention": "OPENMM_FULL_K_HALF_ENERGY",
        "bond_coefficient_unit": "kcal/mol/angstrom^2", "angle_coefficient_unit": "kcal/mol/radian^2",
        "bond_equilibrium_unit": "angstrom", "angle_equilibrium_unit": "radian",
        "bond_uses_periodic_boundary_conditions": False, "angle_uses_periodic_boundary_conditions": False,
        "bond_count": 0, "angle_count": 0, "contract_sha256": ""}
    d["bonds"][1]["k"] = 2.0e-30
    return prep.seal(d)


def test_harmonic_lowering_small_document(pq):
    d = _harmonic_doc()
    t, _, _ = _same(pq, d)
    assert t.bonds["k"].tolist() == [300.0, np.float32(1.0e-30)]
    assert t.angles["force_k"].tolist() == [50.0]


@pytest.mark.parametrize("field,value", [
    ("bond_coefficient_unit", "kJ/mol/nm^2"), ("angle_equilibrium_unit", "degree"),
    ("bond_uses_periodic_boundary_conditions", True), ("schema_version", 2), ("source_provider", "  "),
    ("bond_convention", "HALF_K"), ("bond_count", 3)])
def test_harmonic_contract_field_refused(pq, field, value):
    d = _harmonic_doc()
    d["harmonic_parameter_contract"][field] = value
    h = d["harmonic_parameter_contract"]
    if field != "bond_count":
        h["contract_sha256"] = prep.harmonic_contract_digest(h)
    _, want, got = _same(pq, d)
    assert want and got


def test_harmonic_contract_digest_and_unknown_field(pq):
    d = _harmonic_doc()
    d["harmonic_parameter_contract"]["contract_sha256"] = "0" * 64
    _, want, got = _same(pq, d)
    assert "digest mismatch" in want and "digest mismatch" in got
    d = _harmonic_doc()
    d["harmonic_parameter_contract"]["note"] = "x"
    with pytest.raises(pq.PrismQError) as e:  # serde(deny_unknown_fields)
        _ingest(pq, d)
    assert "unknown field" in str(e.value)


def test_harmonic_coefficient_underflow_refused(pq):
    d = _harmonic_doc()
    d["bonds"][1]["k"] = 1.0e-46  # x 0.5 underflows float32 to 0
    prep.seal(d)
    _, want, got = _same(pq, d)
    assert want and "not representable" in got


def test_contract_digest_uses_python_canonical_escapes(pq):
    """Non-ASCII provider text is hashed with \\u escapes (ensure_ascii)."""
    d = _harmonic_doc()
    h = d["harmonic_parameter_contract"]
    h["source_provider"] = "OpenMM/8.1 é中\U0001f600 \"q\" \\ \t"
    h["contract_sha256"] = prep.harmonic_contract_digest(h)
    _same(pq, d)


@pytest.mark.parametrize("text", ['{"n_atoms": 5', '{"a": 01}', '{"a": "\\x"}', '{"a": 1} x', '[1, 2,]', '',
                                  '{"a": "\\ud800"}', '{"a": 1e}', '{"a": -}', '{"a": "\u0001"}'])
def test_malformed_json_refused(pq, text):
    with pytest.raises(pq.PrismQError) as e:
        pq.Topology.from_prep_json(text.encode() if text else b" ")
    assert e.value.status == 1


def test_options_default_and_struct_sizes(pq):
    L = pq.load()
    o = pq.PrepOptionsStruct()
    L.prismq_prep_options_default(ctypes.byref(o))
    assert (o.apply_hmr, o.require_harmonic_contract, o.require_exceptions, o.hmr_factor) == (1, 1, 1, 3.0)
    assert ctypes.sizeof(pq.PrepOptionsStruct) == 24 and ctypes.sizeof(pq.PrepReportStruct) == 48


def test_canonical_form_matches_python(doc):
    h = doc["harmonic_parameter_contract"]
    body = {k: v for k, v in h.items() if k != "contract_sha256"}
    assert prep.canonical(body) == json.dumps(body, sort_keys=True, separators=(",", ":")).encode()
    assert hashlib.sha256(prep.canonical(body)).hexdigest() == h["contract_sha256"]


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_ingested_system_forces_and_trajectory(gpu, orc, doc):
    """The ingested topology runs on the device exactly like the builder's."""
    t = gpu.Topology.from_prep_json(str(FIXTURE))
    b = gpu.Topology.polyala(2, 4, seed=11)
    p = gpu.Params()
    ea, eb = gpu.NhsAmberFusedEngine(t, p), gpu.NhsAmberFusedEngine(b, p)
    pa, fa, xa = ea.compute_forces()
    pb, fb, xb = eb.compute_forces()
    assert np.array_equal(xa, xb) and pa == pb
    o = orc.OracleSystem(t.struct(), dt=p.dt, temperature=p.temperature, gamma=p.gamma, cutoff=p.cutoff,
                         max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed, stream=p.stream)
    f64, e64 = o.forces_f64()
    assert rel_rms(fa, f64) <= 1e-5
    assert abs(pa - e64.sum()) <= 1e-6 * abs(e64).sum()
    ea.run(200)
    eb.run(200)
    assert np.array_equal(ea.get_positions(), eb.get_positions())
    assert np.array_equal(ea.get_velocities(), eb.get_velocities())
    ea.close()
    eb.close()
