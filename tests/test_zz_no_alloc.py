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


def _run(pq, fn, pos: np.ndarray, row_cap: int = 1024):
    import torch

    n = len(pos)
    d_xyz = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1)).cuda()
    d_rows = torch.full((n, row_cap), -7, dtype=torch.int32, device="cuda")
    d_cnt = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(d_xyz.data_ptr(), n, 12.0, row_cap, d_rows.data_ptr(), d_cnt.data_ptr(), None)
    assert rc == 0, pq.load().prismq_last_error()
    return d_rows.cpu().numpy(), d_cnt.cpu().numpy()


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
