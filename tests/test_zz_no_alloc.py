"""GPU: the allocation-free neighbour-row entry point.

prismq_neighbor_rows_noalloc serves callers that cannot allocate device memory
while they run (a serving process that reserves all of its HBM up front, or a
loop whose allocator policy forbids cudaMalloc/cudaFree after start-up).  The
caller owns every buffer; the entry point's own cell lists sit in a fixed
file-scope device array.  Its pair set must equal the existing entry point's
(prismq_build_neighbors, complete mode) exactly — integer output, bit-exact —
on two calls in a row, so the shared scratch is shown to be reset between calls.
This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(pq):
    L = pq.load()
    fn = L.prismq_neighbor_rows_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _rows_to_pairs(rows: np.ndarray, counts: np.ndarray) -> np.ndarray:
    out = []
    for i, c in enumerate(counts):
        assert c >= 0
        for j in rows[i, :c]:
            if j > i:
                out.append((i, int(j)))
    return np.array(sorted(out), dtype=np.int32).reshape(-1, 2)


def _run(pq, fn, pos: np.ndarray, row_cap: int = 1024, expect: int = 0):
    import torch

    n = len(pos)
    d_xyz = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1)).cuda()
    d_rows = torch.full((n, row_cap), -7, dtype=torch.int32, device="cuda")
    d_cnt = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(d_xyz.data_ptr(), n, 12.0, row_cap, d_rows.data_ptr(), d_cnt.data_ptr(), None)
    assert rc == expect, (rc, pq.load().prismq_last_error())
    return d_rows.cpu().numpy(), d_cnt.cpu().numpy()


def _existing_pairs(pq, pos: np.ndarray) -> np.ndarray:
    eng = pq.NhsAmberFusedEngine(pq.Topology.point_cloud(pos), pq.Params())
    want = eng.build_neighbors(pq.NLIST_COMPLETE)
    eng.close()
    return want


def test_noalloc_rows_equal_existing_entry_point_twice(gpu, golden):
    fn = _noalloc(gpu)
    cases = [golden["cloud_2000/pos"], gpu.Topology.polyala(1, 120, seed=21).positions]
    for pos in cases:  # two calls in a row through the same scratch
        rows, cnt = _run(gpu, fn, pos)
        got = _rows_to_pairs(rows, cnt)
        eng = gpu.NhsAmberFusedEngine(gpu.Topology.point_cloud(pos), gpu.Params())
        want = eng.build_neighbors(gpu.NLIST_COMPLETE)
        eng.close()
        assert np.array_equal(got, want)
        # rows hold each pair from both ends
        assert int(cnt.sum()) == 2 * len(want)


def test_noalloc_rejects_sizes_beyond_its_limits(gpu):
    fn = _noalloc(gpu)
    assert fn(None, 70000, 12.0, 64, None, None, None) == 4  # PRISMQ_E_CAPACITY
    assert fn(None, 100, 12.0, 2048, None, None, None) == 4


def test_noalloc_long_thin_cloud_matches_brute_force(gpu, orc):
    """A cloud 6,500 Å long (the grid caps at 1,024 cells on that axis, which
    widens its cells) against the oracle's all-pairs enumeration."""
    rng = np.random.default_rng(77)
    n = 3000
    pos = np.stack([rng.uniform(0.0, 6500.0, n), rng.uniform(0.0, 4.0, n), rng.uniform(0.0, 4.0, n)], axis=1)
    pos = pos.astype(np.float32)
    fn = _noalloc(gpu)
    rows, cnt = _run(gpu, fn, pos)
    got = _rows_to_pairs(rows, cnt)
    want = orc.pairs_brute(pos, 144.0)
    assert len(want) > 1000
    assert np.array_equal(got, want)


def test_noalloc_reports_overflows_and_recovers(gpu, golden):
    """A row longer than row_cap and a cell of more than 512 atoms are reported
    with their status and -1 counts; the next ordinary call through the same
    scratch again equals the existing entry point."""
    fn = _noalloc(gpu)
    cloud = golden["cloud_2000/pos"]
    want = _existing_pairs(gpu, cloud)
    deg = np.bincount(want.reshape(-1), minlength=len(cloud))
    # rows capped at the median row length: the longer rows overflow, the others are whole
    cap = int(np.median(deg))
    rows, cnt = _run(gpu, fn, cloud, row_cap=cap, expect=6)  # PRISMQ_E_NEIGHBOR_OVERFLOW
    assert np.array_equal(cnt == -1, deg > cap)
    assert (deg <= cap).any() and (deg > cap).any()
    for i in np.nonzero(deg <= cap)[0]:
        part = sorted(set(want[want[:, 0] == i, 1]) | set(want[want[:, 1] == i, 0]))
        assert sorted(rows[i, :cnt[i]].tolist()) == part
    # 600 atoms inside one cell
    rng = np.random.default_rng(5)
    dense = rng.uniform(0.0, 1.0, size=(600, 3)).astype(np.float32)
    _, cnt = _run(gpu, fn, dense, expect=5)  # PRISMQ_E_CELL_OVERFLOW
    assert (cnt == -1).all()
    # an ordinary call afterwards
    rows, cnt = _run(gpu, fn, cloud)
    assert np.array_equal(_rows_to_pairs(rows, cnt), want)
