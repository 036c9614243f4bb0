"""CPU: pin the oracle against the reference's own known answers.

* neighbour scheme: golden vectors generated by scripts/physics_refs/neighbor_list.py
  (cell_pairs / brute_pairs) — synthetic_600 must give 94,216 brute-force pairs,
  93,912 kept and 304 missed, none within 10 Å (the reference's REVIEW_BUNDLE.md,
  D-NBL-MISS-10-12);
* Philox4x32-10 Random123 known-answer vectors (rng_streams.py:87-92);
* the 418.4 half-kick (fused_engine.rs:4723-4731);
* COULOMB_CONSTANT 332.0636 against CODATA-derived kcal·Å/(mol·e²).
"""
from __future__ import annotations

import hashlib
import math

import numpy as np
import pytest

CASES = ["synthetic_600", "drift_25x", "cloud_2000"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def test_golden_counts_match_reference_publication(golden):
    c = golden["synthetic_600/counts"]
    assert c[0] == 94216 and c[1] == 93912 and c[2] == 304 and c[3] == 0 and c[4] == 81


@pytest.mark.parametrize("case", CASES)
def test_oracle_ref27_matches_golden(orc, golden, case):
    pos = golden[f"{case}/pos"]
    gpos = golden[f"{case}/grid_pos"]
    r2 = float(golden["cutoff_sq"])
    pairs, occ = orc.pairs_ref27(pos, gpos, r2)
    counts = golden[f"{case}/counts"]
    assert len(pairs) == counts[1]
    assert occ == counts[4]
    assert _sha(pairs) == str(golden[f"{case}/kept_sha256"])


@pytest.mark.parametrize("case", CASES)
def test_oracle_brute_matches_golden_and_missed_set(orc, golden, case):
    pos = golden[f"{case}/pos"]
    r2 = float(golden["cutoff_sq"])
    b = orc.pairs_brute(pos, r2)
    assert _sha(b) == str(golden[f"{case}/brute_sha256"])
    kept, _ = orc.pairs_ref27(pos, golden[f"{case}/grid_pos"], r2)
    bs = set(map(tuple, b.tolist()))
    ks = set(map(tuple, kept.tolist()))
    missed = np.array(sorted(bs - ks), dtype=np.int32).reshape(-1, 2)
    assert np.array_equal(missed, golden[f"{case}/missed"])
    # every missed pair lies beyond the 10 Å potential cutoff (only the buffer is lost)
    d = pos[missed[:, 0]] - pos[missed[:, 1]]
    assert (np.sqrt((d.astype(np.float64) ** 2).sum(1)) > 10.0).all()


def test_empty_and_single_atom_clouds(orc):
    p, occ = orc.pairs_ref27(np.zeros((1, 3), np.float32))
    assert len(p) == 0 and occ == 1
    assert len(orc.pairs_brute(np.zeros((1, 3), np.float32))) == 0
    # coincident atoms are within the list radius (r2 = 0)
    two = np.zeros((2, 3), np.float32)
    p, _ = orc.pairs_ref27(two)
    assert p.tolist() == [[0, 1]]


def test_ref27_cutoff_equality_is_kept(orc):
    # r^2 exactly at 144 must be kept (`!(r2 > cutoff_sq)`)
    pos = np.array([[0, 0, 0], [12, 0, 0], [12.0001, 0, 0]], np.float32)
    pos[2, 0] = 0.0
    pos[2, 1] = 12.0
    p = orc.pairs_brute(pos, 144.0)
    assert [0, 1] in p.tolist() and [0, 2] in p.tolist()
    pos2 = np.array([[0, 0, 0], [np.nextafter(np.float32(12), np.float32(13)), 0, 0]], np.float32)
    assert len(orc.pairs_brute(pos2, 144.0)) == 0


KAT = [  # Random123 kat_vectors, philox4x32 10 rounds (quoted in rng_streams.py)
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(orc, ctr, key, want):
    assert orc.philox(ctr, key) == want


def test_normal_statistics(orc):
    z = np.array([orc.normal3(7, 3, a, s, 1) for a in range(400) for s in range(25)], np.float64).ravel()
    assert abs(z.mean()) < 0.02
    assert abs(z.var() - 1.0) < 0.03
    # fourth moment of a normal is 3
    assert abs((z ** 4).mean() - 3.0) < 0.15


def test_418_4_half_kick_known_answer(orc, pq):
    # one free atom, F = 1 kcal/mol/Å on x, m = 1 amu, dt = 0.001 ps, γ = 0:
    # Δv = 0.5·dt·418.4·F/m = 0.2092 Å/ps after KICK½ (fused_engine.rs:4723-4731)
    topo = pq.Topology(np.zeros((1, 3)), [1.0], [0.0], [3.0], [0.1])
    s = orc.OracleSystem(topo.struct(), dt=0.001, gamma=0.0, temperature=300.0)
    s.set_state(np.zeros((1, 3), np.float32), np.zeros((1, 3), np.float32))
    f = np.array([[1 << 32, 0, 0]], np.int64)  # 1.0 in 2^-32 fixed point
    assert s.phases(2, f, 0) == 0  # post set: KICK½ first; γ = 0 makes OU a no-op
    _, v = s.get_state()
    assert abs(v[0, 0] - 0.2092) < 1e-6 and v[0, 1] == 0.0


def test_coulomb_constant_units():
    # e^2/(4πε0) in kcal·Å/mol from CODATA 2018 constants
    e, eps0, na = 1.602176634e-19, 8.8541878128e-12, 6.02214076e23
    k = e * e / (4 * math.pi * eps0) * 1e10 * na / 4184.0
    assert abs(k - 332.0636) / 332.0636 < 1e-5


def test_oracle_generator_builds_the_library_systems(pq):
    """The CPU legs of the benchmark build their inputs with the oracle's own
    build of the generator; it yields the library's systems bit for bit."""
    from oracle import oracle as orc

    for args, kw in [((1, 120, 9), {}), ((3, 30, 4), {"box_edge": 25.0})]:
        a = pq.Topology.polyala_compact(*args[:2], seed=args[2], **kw)
        b = orc.polyala(*args, **kw)
        for f in ("positions", "masses", "charges", "bonds", "angles", "dihedrals", "exceptions", "exclusions",
                  "clusters"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
    a = pq.Topology.polyala(1, 30, seed=3)
    b = orc.polyala(1, 30, 3, compact=False)
    assert np.array_equal(a.positions, b.positions)
