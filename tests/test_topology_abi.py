"""CPU: the synthetic topology generator, the host-only entry points and the
C ABI surface (every symbol declared in include/prismq_md.h is exported)."""
from __future__ import annotations

import re

import numpy as np
import pytest

from conftest import ROOT


def test_header_symbols_exported(pq):
    text = (ROOT / "include" / "prismq_md.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(prismq_[a-z0-9_]+)\s*\(", text))
    assert len(names) >= 35
    lib = pq.load()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.prismq_abi_version() == 3


def test_no_device_is_reported_not_faked(pq):
    if pq.device_count() > 0:
        pytest.skip("a device is present")
    topo = pq.Topology.polyala(1, 5, seed=1)
    with pytest.raises(pq.PrismQError) as e:
        pq.NhsAmberFusedEngine(topo, pq.Params())
    assert e.value.status == 3  # PRISMQ_E_NO_DEVICE: no CPU fallback


def test_generator_is_deterministic(pq):
    a = pq.Topology.polyala(1, 60, seed=42)
    b = pq.Topology.polyala(1, 60, seed=42)
    c = pq.Topology.polyala(1, 60, seed=43)
    assert np.array_equal(a.positions, b.positions)
    assert not np.array_equal(a.positions, c.positions)
    for f in ("bonds", "angles", "dihedrals", "exceptions", "clusters", "exclusions"):
        assert np.array_equal(getattr(a, f), getattr(b, f))


@pytest.mark.parametrize("nres", [1, 2, 37])
def test_polyala_term_counts(pq, nres):
    t = pq.Topology.polyala(1, nres, seed=5)
    n = 10 * nres
    assert t.n_atoms == n
    assert len(t.bonds) == 10 * nres - 1           # bonds 10R-1
    assert len(t.angles) == 18 * nres - 4          # angles 18R-4
    assert len(t.clusters) == 3 * nres             # NH, CH, CH3 per residue
    assert sum(int(c["n_hydrogens"]) for c in t.clusters) == 5 * nres
    assert abs(float(t.charges.astype(np.float64).sum())) < 1e-4 * nres  # neutral residues


def test_hmr_masses_and_cluster_inverse_masses(pq):
    t = pq.Topology.polyala(1, 8, seed=2)
    for c in t.clusters:
        hs = [h for h in c["hydrogen_atoms"] if h >= 0]
        for h in hs:
            assert abs(t.masses[h] - 3.024) < 1e-5
            assert abs(c["inv_mass_h"] - 1.0 / 3.024) < 1e-6
        central = c["central_atom"]
        assert abs(c["inv_mass_central"] * t.masses[central] - 1.0) < 1e-6
        assert t.masses[central] >= 1.0
    # total mass is conserved by the repartitioning (input.rs:2482-2560)
    raw = {0: 14.01, 1: 1.008, 2: 12.01, 3: 1.008, 4: 12.01, 5: 1.008, 6: 1.008, 7: 1.008, 8: 12.01, 9: 16.00}
    want = sum(raw[a % 10] for a in range(t.n_atoms))
    assert abs(float(t.masses.astype(np.float64).sum()) - want) < 1e-3


def test_exclusions_cover_bonds_angles_and_exceptions(pq):
    t = pq.Topology.polyala(1, 12, seed=9)
    off, ex = t.exclusion_offsets, t.exclusions
    excl = [set(ex[off[a]:off[a + 1]].tolist()) for a in range(t.n_atoms)]
    for b in t.bonds:
        assert b["j"] in excl[b["i"]] and b["i"] in excl[b["j"]]
    for g in t.angles:
        assert g["k"] in excl[g["i"]]
    bonded13 = {(min(g["i"], g["k"]), max(g["i"], g["k"])) for g in t.angles}
    bonded12 = {(min(b["i"], b["j"]), max(b["i"], b["j"])) for b in t.bonds}
    for e in t.exceptions:
        p = (min(e["i"], e["j"]), max(e["i"], e["j"]))
        assert p not in bonded12 and p not in bonded13
        assert e["j"] in excl[e["i"]]
        qi, qj = t.charges[e["i"]], t.charges[e["j"]]
        assert abs(e["charge_product"] - qi * qj / 1.2) < 1e-5
        assert abs(e["sigma"] - 0.5 * (t.lj_sigma[e["i"]] + t.lj_sigma[e["j"]])) < 1e-5


def test_generator_geometry_has_ideal_constraints_and_no_clash(pq):
    t = pq.Topology.polyala(1, 50, seed=4)
    p = t.positions.astype(np.float64)
    for c in t.clusters:
        for h, L in zip(c["hydrogen_atoms"], c["bond_lengths"]):
            if h >= 0:
                d = np.linalg.norm(p[h] - p[c["central_atom"]])
                assert abs(d - L) < 1e-4
    from scipy.spatial import cKDTree

    tree = cKDTree(p)
    close = tree.query_pairs(0.9)
    assert not close


def test_host_noise_matches_oracle_bit_for_bit(pq, orc):
    for atom in range(0, 5000, 97):
        for step in (0, 1, 12345, (1 << 40) + 3):
            for purpose in (1, 2):
                a = pq.debug_noise(0x1234, 77, atom, step, purpose)
                b = orc.normal3(0x1234, 77, atom, step, purpose)
                assert a.tobytes() == b.tobytes()


def test_box_mode_keeps_chains_in_their_cells(pq):
    t = pq.Topology.polyala(4, 20, seed=3, box_edge=80.0)
    p = t.positions
    assert p.min() >= -1e-3
    assert t.n_atoms == 800


def _nonbonded_min_distance(t) -> float:
    """Closest pair of atoms that are more than three bonds apart."""
    from scipy.spatial import cKDTree

    p = t.positions.astype(np.float64)
    pairs = cKDTree(p).query_pairs(2.5, output_type="ndarray")
    if len(pairs) == 0:
        return 99.0
    off, lst = t.exclusion_offsets, t.exclusions
    keep = np.array([b not in lst[off[a]:off[a + 1]] for a, b in pairs])
    if not keep.any():
        return 99.0
    d = np.linalg.norm(p[pairs[keep, 0]] - p[pairs[keep, 1]], axis=1)
    return float(d.min())


def _bond_errors(t):
    p = t.positions.astype(np.float64)
    b = t.bonds
    r = np.linalg.norm(p[b["j"]] - p[b["i"]], axis=1)
    heavy = np.abs(r - b["r0"]) / b["r0"]
    c = t.clusters
    h_err = 0.0
    for k in range(3):
        h = c["hydrogen_atoms"][:, k]
        ok = h >= 0
        rr = np.linalg.norm(p[h[ok]] - p[c["central_atom"][ok]], axis=1)
        h_err = max(h_err, float(np.max(np.abs(rr - c["bond_lengths"][ok, k]) / c["bond_lengths"][ok, k])))
    return float(heavy.max()), h_err


def test_compact_globule_has_the_configured_size(pq):
    """2,500 atoms collapsed into a 40 Å globule (0.0746 atoms/Å^3) with no
    clash: atoms more than three bonds apart stay >= 1.5 Å apart, bonds keep
    their lengths and the hydrogens sit on their constraint lengths."""
    st = {}
    t = pq.Topology.polyala_compact(1, 250, seed=5, stats=st)
    p = t.positions.astype(np.float64)
    assert t.n_atoms == 2500
    ext = p.max(axis=0) - p.min(axis=0)
    assert ext.max() <= 40.5, ext
    rg = float(np.sqrt(((p - p.mean(axis=0)) ** 2).sum(axis=1).mean()))
    assert 13.5 <= rg <= 16.5, rg
    assert st["max_outside"] < 0.1 and st["max_overlap"] < 0.11
    assert _nonbonded_min_distance(t) >= 1.5
    heavy, h = _bond_errors(t)
    assert heavy < 0.05 and h < 5e-6  # float32 rounding of the coordinates
    # same chain, same bonded terms as the grown chain of the same seed
    g = pq.Topology.polyala(1, 250, seed=5)
    for f in ("bonds", "angles", "dihedrals", "exceptions", "clusters", "exclusions", "charges", "masses"):
        assert np.array_equal(getattr(t, f), getattr(g, f)), f


def test_compact_box_packs_every_chain_inside(pq):
    """Chains packed into one cube (the 40-chain, 110 Å system at a smaller
    size: 4 chains of 50 residues in a 29.9 Å cube, 0.0749 atoms/Å^3)."""
    edge = 29.9
    st = {}
    t = pq.Topology.polyala_compact(4, 50, seed=8, box_edge=edge, stats=st)
    p = t.positions.astype(np.float64)
    ext = p.max(axis=0) - p.min(axis=0)
    assert ext.max() <= edge + 0.25, ext
    assert ext.min() >= edge - 3.0, ext
    assert _nonbonded_min_distance(t) >= 1.5
    heavy, h = _bond_errors(t)
    assert heavy < 0.05 and h < 5e-6  # float32 rounding of the coordinates


def test_compact_generator_is_deterministic(pq):
    a = pq.Topology.polyala_compact(1, 40, seed=42)
    b = pq.Topology.polyala_compact(1, 40, seed=42)
    c = pq.Topology.polyala_compact(1, 40, seed=43)
    assert np.array_equal(a.positions, b.positions)
    assert not np.array_equal(a.positions, c.positions)
