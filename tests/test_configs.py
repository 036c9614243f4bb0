"""GPU parity at the sizes and densities of the benchmark configurations:

  config 1  40 chains of 250 residues (100,000 atoms) packed in a 110 Å cube
  config 2  the 256-system batch: chains of 50–800 residues, each collapsed
            into a globule at 0.0746 atoms/Å^3 (2,500 atoms in 40 Å)

Bars as for the small systems: the COMPLETE pair set bit-exact against the
oracle's all-pairs enumeration, REF27 bit-exact against the oracle's
restatement of the reference scheme, forces within 1e-5 relative RMS and
potential energies within 1e-6 of the FP64 oracle — for config 2 on every
one of the 256 systems, at the built positions and again after 100 steps.
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6
SEED = 20261203  # the benchmark's seed


@pytest.fixture(scope="module")
def config1(pq):
    return pq.Topology.polyala_compact(40, 250, seed=SEED, box_edge=110.0)


def _oracle(orc, topo, p, **kw):
    return orc.OracleSystem(topo.struct(), dt=p.dt, temperature=p.temperature, gamma=p.gamma, cutoff=p.cutoff,
                            max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed,
                            stream=p.stream, **kw)


def test_config1_pair_sets_and_forces(gpu, orc, config1):
    t = config1
    assert t.n_atoms == 100_000
    ext = t.positions.max(axis=0) - t.positions.min(axis=0)
    assert ext.max() <= 110.3, ext
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(t, p)
    o = _oracle(orc, t, p)
    off, lst = o.ref_exclusions()
    got = eng.build_neighbors(gpu.NLIST_COMPLETE)
    want = orc.pairs_brute(t.positions, 144.0, off, lst)
    assert len(want) > 20_000_000
    assert np.array_equal(got, want)
    del got, want
    want_ref, occ = orc.pairs_ref27(t.positions, t.positions, 144.0, off, lst)
    assert np.array_equal(eng.build_neighbors(gpu.NLIST_REF27), want_ref)
    del want_ref
    pe, f, _ = eng.compute_forces()
    f64, e64 = o.forces_f64(os.cpu_count() or 1)
    assert rel_rms(f, f64) <= FORCE_RTOL
    assert abs(pe - e64.sum()) <= ENERGY_RTOL * abs(e64).sum()
    comp = eng.energy_components()
    for k in range(5):
        assert abs(comp[k] - e64[k]) <= ENERGY_RTOL * max(abs(e64[k]), 1.0), (k, comp[k], e64[k])
    # a short trajectory stays finite and keeps the cube packed
    eng.step(40)
    x = eng.get_positions()
    assert np.isfinite(x).all()
    o.close()
    eng.close()


def _batch256_topologies(pq):
    rng = np.random.default_rng(SEED)
    res = np.exp(rng.uniform(math.log(50), math.log(800), size=256))
    sizes = [int(round(r)) for r in res]

    def one(i):
        return pq.Topology.polyala_compact(1, sizes[i], seed=SEED + 7919 * i)

    with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 4)) as ex:
        return list(ex.map(one, range(256)))


def test_batch256_forces_vs_fp64_every_system(gpu, orc):
    topos = _batch256_topologies(gpu)
    atoms = sum(t.n_atoms for t in topos)
    assert 600_000 < atoms < 800_000
    b = gpu.Batch(atoms + 64 * len(topos), len(topos))
    params = [gpu.Params(stream=i) for i in range(len(topos))]
    slots = [b.add_system(t, p) for t, p in zip(topos, params)]
    threads = os.cpu_count() or 1

    def check(positions):
        errs = []
        for k, s in enumerate(slots):
            e = b.energy(s)  # one evaluation refreshes every resident system's forces
            f = b.forces_f64(s)
            t = topos[k]
            tt = gpu.Topology(positions[k], t.masses, t.charges, t.lj_sigma, t.lj_epsilon, t.bonds, t.angles,
                              t.dihedrals, t.exceptions, t.exclusion_offsets, t.exclusions, t.clusters)
            o = _oracle(orc, tt, params[k])
            f64, e64 = o.forces_f64(threads)
            o.close()
            errs.append(rel_rms(f, f64))
            assert abs(e[:5].sum() - e64.sum()) <= ENERGY_RTOL * abs(e64).sum(), (k, e[:5], e64)
        errs = np.array(errs)
        assert (errs <= FORCE_RTOL).all(), (int(errs.argmax()), float(errs.max()))
        return errs

    check([t.positions for t in topos])
    b.step(100)
    for s in slots:
        assert b.status(s) == 0
    check([b.get_state(s)[0] for s in slots])
    b.close()
