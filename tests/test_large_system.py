"""A system of 20,000 atoms, above the size at which the cell sort moves from
the system's control block to grid-wide kernels.  Bars as for small systems:
pair sets bit-exact against brute force (COMPLETE) and the reference scheme
(REF27), forces within 1e-5 relative RMS of the FP64 oracle, repeat runs
bit-identical, and the same system in a batch with small ones identical to
its solo run."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(pq):
    t = pq.Topology.polyala(2, 1000, seed=21)
    assert t.n_atoms >= 16384
    return t


def _oracle(orc, topo, p):
    return orc.OracleSystem(topo.struct(), dt=p.dt, temperature=p.temperature, gamma=p.gamma, cutoff=p.cutoff,
                            max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed, stream=p.stream)


def test_large_system_pair_sets(gpu, orc, big):
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(big, p)
    o = _oracle(orc, big, p)
    off, lst = o.ref_exclusions()
    want_all = orc.pairs_brute(big.positions, 144.0, off, lst)
    assert np.array_equal(eng.build_neighbors(gpu.NLIST_COMPLETE), want_all)
    want_ref, _ = orc.pairs_ref27(big.positions, big.positions, 144.0, off, lst)
    assert np.array_equal(eng.build_neighbors(gpu.NLIST_REF27), want_ref)
    eng.close()


def test_large_system_forces_vs_fp64(gpu, orc, big):
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(big, p)
    pe, f, _ = eng.compute_forces()
    f64, e64 = _oracle(orc, big, p).forces_f64()
    assert rel_rms(f, f64) <= 1e-5
    assert abs(pe - e64.sum()) <= 1e-6 * abs(e64).sum()
    eng.close()


def test_large_system_runs_repeat_and_batch_identically(gpu, big):
    a = gpu.NhsAmberFusedEngine(big, gpu.Params(stream=5))
    b = gpu.NhsAmberFusedEngine(big, gpu.Params(stream=5))
    a.step(45)
    for _ in range(3):
        b.step(15)
    assert np.array_equal(a.get_positions(), b.get_positions())
    assert np.array_equal(a.get_velocities(), b.get_velocities())
    small = gpu.Topology.polyala(1, 30, seed=2)
    bat = gpu.Batch(max_atoms=big.n_atoms + 1024, max_systems=4)
    s0 = bat.add_system(small, gpu.Params(stream=1))
    s1 = bat.add_system(big, gpu.Params(stream=5))
    bat.step(45)
    x, v = bat.get_state(s1)
    assert np.array_equal(x, a.get_positions()) and np.array_equal(v, a.get_velocities())
    e = gpu.NhsAmberFusedEngine(small, gpu.Params(stream=1))
    e.step(45)
    x, v = bat.get_state(s0)
    assert np.array_equal(x, e.get_positions()) and np.array_equal(v, e.get_velocities())
    for s in (a, b, e):
        s.close()
    bat.close()
