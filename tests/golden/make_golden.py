"""Generate tests/golden/neighbor_golden.npz from the reference's own CPU check.

Imports scripts/physics_refs/neighbor_list.py from a Prism-Q checkout (path
given as argv[1]) and records, for seeded point clouds, the pair set of the
reference cell scheme (cell_pairs) and of brute force (brute_pairs) at the
reference list radius (r^2 <= (10 Å)^2 * 1.44):

  synthetic_600   the reference's synthetic_cloud() (600 atoms, seed 20261023)
  drift_25x       the same cloud moved +25 Å along x, grid fixed from the
                  original positions (the clamping case of check_neighbor_cells)
  cloud_2000      synthetic_cloud(n=2000, radius=17.0, seed=7)

Stored per case: float32 positions, the grid positions, counts, the maximum
cell occupancy, the SHA-256 of the sorted int32 (i<j) pair arrays, and the
missed pairs (brute minus kept) in full.  Run once in a container that has the
reference checkout; the fixture is committed and no test reads the reference.
"""
from __future__ import annotations

import hashlib
import importlib.util
import pathlib
import sys

import numpy as np


def _load(ref_root: pathlib.Path):
    p = ref_root / "scripts" / "physics_refs" / "neighbor_list.py"
    spec = importlib.util.spec_from_file_location("ref_neighbor_list", p)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ref_neighbor_list"] = mod
    spec.loader.exec_module(mod)
    return mod


def pairs_array(s: set) -> np.ndarray:
    a = np.array(sorted(s), dtype=np.int32).reshape(-1, 2)
    return a


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def main(ref_root: str) -> None:
    nl = _load(pathlib.Path(ref_root))
    F32 = np.float32
    cutoff_sq = F32(F32(10.0) * F32(10.0)) * F32(1.44)
    base = nl.synthetic_cloud()
    cases = {
        "synthetic_600": (base, base),
        "drift_25x": (base + np.array([25.0, 0.0, 0.0]), base),
        "cloud_2000": (nl.synthetic_cloud(n=2000, radius=17.0, seed=7),) * 2,
    }
    out = {"cutoff_sq": np.float32(cutoff_sq)}
    for name, (pos, grid_pos) in cases.items():
        origin, n = nl.grid_from_bbox(grid_pos)
        kept, occ = nl.cell_pairs(pos, origin, n, cutoff_sq)
        ref, _ = nl.brute_pairs(pos, cutoff_sq)
        k = pairs_array(kept)
        b = pairs_array(ref)
        missed = pairs_array(ref - kept)
        extra = pairs_array(kept - ref)
        out[f"{name}/pos"] = pos.astype(np.float32)
        out[f"{name}/grid_pos"] = grid_pos.astype(np.float32)
        out[f"{name}/counts"] = np.array([len(b), len(k), len(missed), len(extra), occ], dtype=np.int64)
        out[f"{name}/grid_dims"] = np.asarray(n, dtype=np.int64)
        out[f"{name}/kept_sha256"] = np.array(sha(k))
        out[f"{name}/brute_sha256"] = np.array(sha(b))
        out[f"{name}/missed"] = missed
        print(name, "brute", len(b), "kept", len(k), "missed", len(missed), "extra", len(extra), "occ", occ)
    dst = pathlib.Path(__file__).with_name("neighbor_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout root>")
    main(sys.argv[1])
