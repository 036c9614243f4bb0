"""Precision study: the FP32 production path against an FP64-everywhere run.

The FP64 run keeps positions, velocities, forces, LJ parameters and every
integrator phase in double (same phase order, same injected Philox noise);
only the cell and neighbour-row kernels read its FP32 rounding.  Bars:
  * FP64 forces vs the FP64 oracle (same pair-inclusion rule, r^2 in double):
    relative RMS <= 1e-10, energies within 1e-10 relative;
  * FP32 production forces vs the FP64 run at the same positions: relative
    RMS <= 1e-5 (the production bar);
  * SHAKE at tolerance 1e-6 on |r^2-L^2|/L^2 in the FP64 run: every X-H bond
    length within 1e-6 relative along the trajectory;
  * repeat runs bit-identical in both precisions;
  * the virial W_ab = sum_i x_a F_b equals the same sum over the oracle's
    FP64 forces.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _oracle(orc, topo, p):
    return orc.OracleSystem(topo.struct(), dt=p.dt, temperature=p.temperature, gamma=p.gamma, cutoff=p.cutoff,
                            max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed,
                            stream=p.stream)


def _bond_rel_err(topo, x):
    errs = []
    for c in topo.clusters:
        for h, L in zip(c["hydrogen_atoms"], c["bond_lengths"]):
            if h >= 0:
                r = np.linalg.norm(x[h] - x[c["central_atom"]])
                errs.append(abs(r - float(L)) / float(L))
    return max(errs)


@pytest.mark.parametrize("nchains,nres,box", [(1, 40, 0.0), (1, 250, 0.0), (3, 60, 70.0)])
def test_fp64_forces_match_fp64_oracle(gpu, orc, nchains, nres, box):
    topo = gpu.Topology.polyala(nchains, nres, seed=7, box_edge=box)
    p = gpu.Params(precision=gpu.PRECISION_FP64)
    eng = gpu.NhsAmberFusedEngine(topo, p)
    pe, _, _ = eng.compute_forces()
    f = eng.get_forces_f64()
    f64, e64 = _oracle(orc, topo, p).forces_f64(incl64=True)
    assert rel_rms(f, f64) <= 1e-10
    assert abs(pe - e64.sum()) <= 1e-10 * abs(e64).sum()
    comp = eng.energy_components()
    for k in range(5):
        assert abs(comp[k] - e64[k]) <= 1e-10 * max(abs(e64[k]), 1.0), (k, comp[k], e64[k])
    # virial: sum_i x_a F_b over the oracle's forces at the same positions
    w = eng.virial()
    w_ref = topo.positions.astype(np.float64).T @ f64
    assert np.abs(w - w_ref).max() <= 1e-9 * np.abs(w_ref).max()
    eng.close()


def test_fp32_forces_vs_fp64_run(gpu, ala250):
    e32 = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    e64 = gpu.NhsAmberFusedEngine(ala250, gpu.Params(precision=gpu.PRECISION_FP64))
    e32.compute_forces()
    e64.compute_forces()
    err = rel_rms(e32.get_forces_f64(), e64.get_forces_f64())
    assert 0.0 < err <= 1e-5  # FP32 arithmetic differs, within the production bar
    # the FP32 virial is the FP64 reduction of the FP32 forces
    w32 = e32.virial()
    x = ala250.positions.astype(np.float64)
    assert np.abs(w32 - x.T @ e32.get_forces_f64()).max() <= 1e-9 * np.abs(w32).max()
    e32.close()
    e64.close()


def test_fp64_shake_holds_bonds_to_1e6(gpu, ala250):
    p = gpu.Params(precision=gpu.PRECISION_FP64, shake_tol=1e-6, rattle_tol=1e-7)
    eng = gpu.NhsAmberFusedEngine(ala250, p)
    for _ in range(4):
        eng.step(50)
        x, _ = eng.get_state_f64()
        assert _bond_rel_err(ala250, x) <= 1e-6
    eng.close()


def test_fp32_constraint_check_in_fp64(gpu, ala250):
    # FP64 residuals and multipliers at the reference tolerances: the run holds
    # the reference's bond bar and tracks the FP32-checked run closely
    a = gpu.NhsAmberFusedEngine(ala250, gpu.Params(constraint_check_fp64=True))
    b = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    a.step(100)
    b.step(100)
    xa, xb = a.get_positions().astype(np.float64), b.get_positions().astype(np.float64)
    assert _bond_rel_err(ala250, xa) <= 0.6e-4  # |r-L|/L <= tol/2 for tol 1e-4 on r^2 (+ rounding)
    assert np.sqrt(((xa - xb) ** 2).sum(axis=1).mean()) < 1e-2
    a.close()
    b.close()


def test_mixed_constraint_checks_in_one_batch(gpu, ala40):
    # FP32-checked and FP64-checked systems share a batch (two integrate
    # passes per step); each matches its own run alone
    pa, pb = gpu.Params(stream=1), gpu.Params(stream=2, constraint_check_fp64=True)
    alone = []
    for p in (pa, pb):
        e = gpu.NhsAmberFusedEngine(ala40, p)
        e.step(120)
        alone.append((e.get_positions(), e.get_velocities()))
        e.close()
    b = gpu.Batch(max_atoms=2 * ala40.n_atoms + 128, max_systems=2)
    sa, sb = b.add_system(ala40, pa), b.add_system(ala40, pb)
    b.step(120)
    for s, (x, v) in zip((sa, sb), alone):
        xs, vs = b.get_state(s)
        assert np.array_equal(xs, x) and np.array_equal(vs, v)
    b.close()


def test_fp64_runs_are_repeatable_and_track_fp32(gpu, ala250):
    p64 = gpu.Params(precision=gpu.PRECISION_FP64)
    a = gpu.NhsAmberFusedEngine(ala250, p64)
    b = gpu.NhsAmberFusedEngine(ala250, p64)
    c = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    a.step(60)
    b.step(25)
    b.step(35)
    c.step(60)
    xa, va = a.get_state_f64()
    xb, vb = b.get_state_f64()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    # same noise, same start: the FP32 run stays close over 60 steps
    xc = c.get_positions().astype(np.float64)
    assert np.sqrt(((xa - xc) ** 2).sum(axis=1).mean()) < 1e-2
    for e in (a, b, c):
        e.close()


def test_fp64_batch_rejects_fp32_systems(gpu, ala40):
    b = gpu.Batch(max_atoms=ala40.n_atoms + 64, max_systems=1, precision=gpu.PRECISION_FP64)
    with pytest.raises(gpu.PrismQError) as e:
        b.add_system(ala40, gpu.Params())
    assert e.value.status == 1
    b.close()
