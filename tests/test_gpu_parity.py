"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the
reference's golden pair sets.

Bars (stated per test):
  * neighbour pair sets: bit-exact (REF27 vs the reference scheme, COMPLETE vs
    brute force) — integer/index work keeps its arithmetic;
  * forces: relative RMS <= 1e-5 against the FP64 oracle; potential energy
    within 1e-6 relative;
  * integrator phases: bit-exact against the oracle given the device forces;
  * whole steps: bit-exact against the oracle's phases fed the device forces.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def _oracle(orc, topo, params, **kw):
    return orc.OracleSystem(topo.struct(), dt=params.dt, temperature=params.temperature, gamma=params.gamma,
                            cutoff=params.cutoff, max_iter=params.max_constraint_iter,
                            com_interval=params.com_interval, seed=params.seed, stream=params.stream, **kw)


@pytest.mark.parametrize("case", ["synthetic_600", "drift_25x", "cloud_2000"])
def test_pair_sets_match_reference_golden(gpu, golden, case):
    import hashlib

    pos, gpos = golden[f"{case}/pos"], golden[f"{case}/grid_pos"]
    topo = gpu.Topology.point_cloud(gpos)
    eng = gpu.NhsAmberFusedEngine(topo, gpu.Params())
    eng.set_positions(pos)  # the reference grid stays fixed at the construction positions
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()
    ref = eng.build_neighbors(gpu.NLIST_REF27)
    assert len(ref) == golden[f"{case}/counts"][1]
    assert sha(ref) == str(golden[f"{case}/kept_sha256"])
    comp = eng.build_neighbors(gpu.NLIST_COMPLETE)
    assert len(comp) == golden[f"{case}/counts"][0]
    assert sha(comp) == str(golden[f"{case}/brute_sha256"])
    eng.close()


def test_pair_sets_polyala_with_exclusions(gpu, orc, ala250):
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(ala250, p)
    o = _oracle(orc, ala250, p)
    off, lst = o.ref_exclusions()
    want_ref, _ = orc.pairs_ref27(ala250.positions, ala250.positions, 144.0, off, lst)
    want_all = orc.pairs_brute(ala250.positions, 144.0, off, lst)
    got_ref = eng.build_neighbors(gpu.NLIST_REF27)
    got_all = eng.build_neighbors(gpu.NLIST_COMPLETE)
    assert np.array_equal(got_ref, want_ref)
    assert np.array_equal(got_all, want_all)
    # REF27 ⊂ COMPLETE, and every pair the reference scheme misses lies beyond 10 Å
    s_ref = set(map(tuple, got_ref.tolist()))
    s_all = set(map(tuple, got_all.tolist()))
    assert s_ref <= s_all
    missed = np.array(sorted(s_all - s_ref)).reshape(-1, 2)
    if len(missed):
        d = ala250.positions[missed[:, 0]].astype(np.float64) - ala250.positions[missed[:, 1]]
        assert (np.linalg.norm(d, axis=1) > 10.0).all()
    eng.close()


@pytest.mark.parametrize("nchains,nres,box", [(1, 40, 0.0), (1, 250, 0.0), (3, 60, 70.0)])
def test_forces_and_energy_vs_fp64_oracle(gpu, orc, nchains, nres, box):
    topo = gpu.Topology.polyala(nchains, nres, seed=7, box_edge=box)
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(topo, p)
    pe, f, fx = eng.compute_forces()
    o = _oracle(orc, topo, p)
    f64, e64 = o.forces_f64()
    assert rel_rms(f, f64) <= FORCE_RTOL
    assert abs(pe - e64.sum()) <= ENERGY_RTOL * abs(e64).sum()
    comp = eng.energy_components()
    for k in range(5):
        assert abs(comp[k] - e64[k]) <= ENERGY_RTOL * max(abs(e64[k]), 1.0), (k, comp[k], e64[k])
    # float and fixed-point outputs agree: f = fixed * 2^-32
    assert np.array_equal(f, (fx.astype(np.float32) * np.float32(2.0 ** -32)))
    # the FP32 restatement of the reference gather lands within the same bar
    f32, _ = o.forces_ref_f32()
    assert rel_rms(f, f32) <= FORCE_RTOL
    eng.close()


def test_forces_are_bitwise_deterministic(gpu, ala250):
    eng = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    a = eng.compute_forces()[2]
    b = eng.compute_forces()[2]
    eng2 = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    c = eng2.compute_forces()[2]
    assert np.array_equal(a, b) and np.array_equal(a, c)
    eng.close()
    eng2.close()


@pytest.mark.parametrize("gamma", [1.0, 0.0])
def test_phase_sets_bit_exact(gpu, orc, ala40, gamma):
    p = gpu.Params(gamma=gamma)
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    o = _oracle(orc, ala40, p)
    for step in (0, 3, 101):
        x, v = eng.get_positions(), eng.get_velocities()
        _, _, fx = eng.compute_forces()
        o.set_state(x, v)
        eng.debug_phases(gpu.PHASES_PRE, step)
        assert o.phases(1, fx, step) == 0
        xg, vg = eng.get_positions(), eng.get_velocities()
        xo, vo = o.get_state()
        assert np.array_equal(xg, xo) and np.array_equal(vg, vo)
        _, _, fx = eng.compute_forces()
        eng.debug_phases(gpu.PHASES_POST, step)
        assert o.phases(2, fx, step) == 0
        xg, vg = eng.get_positions(), eng.get_velocities()
        xo, vo = o.get_state()
        assert np.array_equal(xg, xo) and np.array_equal(vg, vo)
    eng.close()


@pytest.mark.parametrize("start_step", [0, 7, 100])
def test_full_step_bit_exact_with_device_forces(gpu, orc, ala40, start_step):
    """One production step (fused kernels, graph) equals the oracle's reference
    phase order fed the device forces F(x_n) and F(x_n+1); start 100 includes
    the COM removal at the start of the step."""
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    eng.step(3)  # leave the initial state
    eng.set_timestep(start_step)
    x, v = eng.get_positions(), eng.get_velocities()
    _, _, f_n = eng.compute_forces()
    eng.step(1)
    _, _, f_np1 = eng.compute_forces()
    o = _oracle(orc, ala40, p)
    o.set_state(x, v)
    if start_step > 0 and start_step % p.com_interval == 0:
        o.com_remove()
    assert o.phases(1, f_n, start_step) == 0
    xo_mid, _ = o.get_state()
    assert o.phases(2, f_np1, start_step) == 0
    xg, vg = eng.get_positions(), eng.get_velocities()
    xo, vo = o.get_state()
    assert np.array_equal(xg, xo_mid) and np.array_equal(xg, xo)
    assert np.array_equal(vg, vo)
    assert eng.timestep == start_step + 1
    eng.close()


def test_trajectory_tracks_reference_cpu_path(gpu, orc, ala40):
    """50 steps of the GPU step vs the oracle's reference step loop (its own FP32
    forces, per-step REF27 list, same injected noise).  The two force
    evaluations differ at ~1e-6 relative, and MD amplifies that difference, so
    the stated tolerance grows with time: after 10 steps max |dx| < 2e-4 Å;
    after 50 steps RMS |dx| < 2e-3 Å and max |dx| < 1e-2 Å."""
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    x, v = eng.get_positions(), eng.get_velocities()
    o = _oracle(orc, ala40, p)
    o.set_state(x, v)
    eng.step(10)
    assert o.run(10) == 0
    d = eng.get_positions().astype(np.float64) - o.get_state()[0]
    assert np.abs(d).max() < 2e-4
    eng.step(40)
    assert o.run(40) == 0
    d = eng.get_positions().astype(np.float64) - o.get_state()[0]
    assert np.sqrt((d ** 2).sum(1).mean()) < 2e-3
    assert np.abs(d).max() < 1e-2
    eng.close()


def _temperature(v, m, n_constraints):
    ke = 0.5 * (m[:, None] * v.astype(np.float64) ** 2).sum() / 418.4
    dof = 3 * len(m) - n_constraints - 3
    return 2.0 * ke / (dof * 0.001987204)


def test_thousand_step_statistics_match_reference_cpu_path(gpu, orc):
    """1,000 steps (4 ps) of the GPU step and of the oracle's reference step loop
    from the same state and noise, on the 2,500-atom globule: trajectories
    decorrelate, so the comparison is statistical — mean kinetic temperature
    over steps 550-1000 within 5% of each other and 8% of the 300 K bath, mean
    potential energy within 3% of the mean total |PE| scale.  At 2,500 atoms
    the instantaneous temperature fluctuates by sqrt(2/3N) = 1.6% and the
    2 ps window holds about two friction times (1/gamma = 1 ps), so the
    difference of the two means has a spread near 1.6% and the 5% bar sits
    three spreads out.  (On a 400-atom chain the spread is near 4%, so a
    change of rounding anywhere in the force sum can carry the two means
    across a 5% bar.)"""
    topo = gpu.Topology.polyala_compact(1, 250, seed=11)
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(topo, p)
    o = _oracle(orc, topo, p)
    o.set_state(eng.get_positions(), eng.get_velocities())
    ncon = int(sum(int(c["n_hydrogens"]) for c in topo.clusters))
    m = topo.masses.astype(np.float64)
    tg, to, eg, eo = [], [], [], []
    for blk in range(20):
        eng.step(50)
        assert o.run(50) == 0
        if blk >= 10:
            tg.append(_temperature(eng.get_velocities(), m, ncon))
            to.append(_temperature(o.get_state()[1], m, ncon))
            eg.append(eng.compute_forces()[0])
            eo.append(o.forces_ref_f32()[1].sum())
    tg, to = np.mean(tg), np.mean(to)
    assert abs(tg - to) / 300.0 < 0.05
    assert abs(tg - 300.0) / 300.0 < 0.08 and abs(to - 300.0) / 300.0 < 0.08
    scale = np.mean(np.abs(eo))
    assert abs(np.mean(eg) - np.mean(eo)) / scale < 0.03
    eng.close()


def test_repeat_runs_are_bit_identical(gpu, ala250):
    a = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    b = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    a.step(137)
    b.step(60)
    b.step(77)  # different call split, same trajectory
    assert np.array_equal(a.get_positions(), b.get_positions())
    assert np.array_equal(a.get_velocities(), b.get_velocities())
    a.close()
    b.close()


def test_every_force_launch_shape_gives_the_same_bits(gpu):
    """The autotuner's launch shapes (registers per thread) change speed
    only: 45 steps of a mixed batch, across list rebuilds, end in the same
    bits under each shape."""
    topos = [gpu.Topology.polyala(1, n, seed=30 + n) for n in (7, 45, 130)]
    states, shapes = [], []
    n_shapes = 1
    v = 0
    while v < n_shapes:
        b = gpu.Batch(max_atoms=2048, max_systems=4)
        slots = [b.add_system(t, gpu.Params(stream=k)) for k, t in enumerate(topos)]
        n_shapes = b.set_force_variant(v)
        b.step(45)
        states.append([b.get_state(s) for s in slots])
        shapes.append(b.tuning())
        b.close()
        v += 1
    keys = {(s["block"], s["min_blocks_per_sm"], s["row_prefetch"]) for s in shapes}
    assert n_shapes >= 2 and len(keys) == n_shapes
    assert {s["atoms_per_block"] for s in shapes} == {32, 64} and {s["row_prefetch"] for s in shapes} == {0, 4}
    for other in states[1:]:
        for (x0, v0), (x1, v1) in zip(states[0], other):
            assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


def test_constraints_hold_along_the_trajectory(gpu, ala250):
    eng = gpu.NhsAmberFusedEngine(ala250, gpu.Params())
    for _ in range(5):
        eng.step(40)
        x = eng.get_positions().astype(np.float64)
        for c in ala250.clusters:
            for h, L in zip(c["hydrogen_atoms"], c["bond_lengths"]):
                if h >= 0:
                    r2 = ((x[h] - x[c["central_atom"]]) ** 2).sum()
                    # SHAKE tolerance of the reference: |r^2 - L^2| / L^2 <= 1e-4 (f32 residual)
                    assert abs(r2 - L * L) / (L * L) <= 1.2e-4
    eng.close()


def test_shake_nonconvergence_is_reported_not_trapped(gpu, ala40):
    p = gpu.Params(max_constraint_iter=1, temperature=600.0)
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    with pytest.raises(gpu.PrismQError) as e:
        eng.step(50)
    assert e.value.status in (7, 8)  # E_SHAKE / E_RATTLE; the context stays usable
    eng2 = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    eng2.step(5)
    eng.close()
    eng2.close()


def test_invalid_topology_rejected_on_host(gpu, ala40):
    bad = gpu.Topology(ala40.positions, ala40.masses, ala40.charges, ala40.lj_sigma, ala40.lj_epsilon,
                       ala40.bonds.copy(), ala40.angles, ala40.dihedrals, ala40.exceptions,
                       ala40.exclusion_offsets, ala40.exclusions, ala40.clusters.copy())
    bad.clusters["inv_mass_h"][0] *= 1.5  # inconsistent with the hydrogen's mass
    with pytest.raises(gpu.PrismQError) as e:
        gpu.NhsAmberFusedEngine(bad, gpu.Params())
    assert e.value.status == 1
    bad2 = gpu.Topology(ala40.positions, ala40.masses, ala40.charges, ala40.lj_sigma, ala40.lj_epsilon,
                        ala40.bonds.copy())
    bad2.bonds["j"][0] = ala40.n_atoms + 5
    with pytest.raises(gpu.PrismQError):
        gpu.NhsAmberFusedEngine(bad2, gpu.Params())
    for per in (0, -2, 65):  # the reference rejects n <= 0; the torsion recurrence bounds n above
        bad3 = gpu.Topology(ala40.positions, ala40.masses, ala40.charges, ala40.lj_sigma, ala40.lj_epsilon,
                            ala40.bonds, ala40.angles, ala40.dihedrals.copy(), ala40.exceptions,
                            ala40.exclusion_offsets, ala40.exclusions, ala40.clusters)
        bad3.dihedrals["periodicity"][3] = per
        with pytest.raises(gpu.PrismQError) as e:
            gpu.NhsAmberFusedEngine(bad3, gpu.Params())
        assert e.value.status == 1 and "periodicity" in str(e.value)


def test_tiny_and_ragged_systems(gpu, orc):
    """Systems of 1, 2 and 3 atoms (partial force groups, warps and cells)
    step beside a 70-atom chain: a lone atom feels exactly zero force; a pair
    and a triple match the FP64 oracle; after 30 steps every state is finite
    and each system equals its solo run."""
    clouds = [np.array([[1.0, 2.0, 3.0]], np.float32),
              np.array([[0.0, 0.0, 0.0], [3.6, 0.5, -0.2]], np.float32),
              np.array([[0.0, 0.0, 0.0], [3.8, 0.0, 0.0], [0.0, 4.1, 0.3]], np.float32)]
    topos = [gpu.Topology.point_cloud(c) for c in clouds] + [gpu.Topology.polyala(1, 7, seed=2)]
    for t in topos[:3]:
        eng = gpu.NhsAmberFusedEngine(t, gpu.Params())
        _, f, fx = eng.compute_forces()
        if t.n_atoms == 1:
            assert not fx.any()
        else:
            f64, _ = _oracle(orc, t, gpu.Params()).forces_f64()
            assert rel_rms(f, f64) <= FORCE_RTOL
        eng.close()
    b = gpu.Batch(max_atoms=1024, max_systems=8)
    slots = [b.add_system(t, gpu.Params(stream=k)) for k, t in enumerate(topos)]
    b.step(30)
    for k, (s, t) in enumerate(zip(slots, topos)):
        x, v = b.get_state(s)
        assert np.isfinite(x).all() and np.isfinite(v).all()
        solo = gpu.Batch(max_atoms=t.n_atoms + 64, max_systems=1)
        ss = solo.add_system(t, gpu.Params(stream=k))
        solo.step(30)
        xs, vs = solo.get_state(ss)
        solo.close()
        assert np.array_equal(x, xs) and np.array_equal(v, vs)
    b.close()


@pytest.mark.parametrize("layout", ["rows", "tiles"])
def test_every_force_launch_shape_gives_the_same_bits_in_each_layout(gpu, layout):
    """Both list layouts, compact chains: each launch shape of the force
    kernel ends 45 steps (across list rebuilds) in the same bits."""
    topos = [gpu.Topology.polyala_compact(1, n, seed=60 + n) for n in (9, 52, 140)]
    lay = gpu.PAIR_ROWS if layout == "rows" else gpu.PAIR_TILES
    states = []
    n_shapes, v = 1, 0
    while v < n_shapes:
        b = gpu.Batch(max_atoms=2048, max_systems=4)
        b.set_pair_layout(lay)
        slots = [b.add_system(t, gpu.Params(stream=k)) for k, t in enumerate(topos)]
        n_shapes = b.set_force_variant(v)
        assert b.pair_layout == lay
        b.step(45)
        states.append([b.get_state(s) for s in slots])
        b.close()
        v += 1
    for other in states[1:]:
        for (x0, v0), (x1, v1) in zip(states[0], other):
            assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


def test_tile_and_row_layouts_hold_the_same_pairs_and_forces(gpu, orc):
    """The cluster-pair tiles and the per-atom rows list the same pairs; their
    forces (FP32 partial sums grouped differently) agree with each other and
    with the FP64 oracle within the force bar, energies within the energy
    bar, and each layout repeats its own bits."""
    topo = gpu.Topology.polyala_compact(1, 300, seed=17)
    p = gpu.Params()
    out = {}
    for name, lay in (("rows", gpu.PAIR_ROWS), ("tiles", gpu.PAIR_TILES)):
        eng = gpu.NhsAmberFusedEngine(topo, p)
        eng.set_pair_layout(lay)
        pairs = eng.build_neighbors(gpu.NLIST_COMPLETE)
        pe, f, fx = eng.compute_forces()
        comp = eng.energy_components()
        _, _, fx2 = eng.compute_forces()
        assert np.array_equal(fx, fx2)
        out[name] = (pairs, pe, f, comp)
        eng.close()
    assert np.array_equal(out["rows"][0], out["tiles"][0])
    off, lst = _oracle(orc, topo, p).ref_exclusions()
    assert np.array_equal(out["tiles"][0], orc.pairs_brute(topo.positions, 144.0, off, lst))
    f64, e64 = _oracle(orc, topo, p).forces_f64()
    for name in ("rows", "tiles"):
        _, pe, f, comp = out[name]
        assert rel_rms(f, f64) <= FORCE_RTOL, name
        assert abs(pe - e64.sum()) <= ENERGY_RTOL * abs(e64).sum(), name
    assert rel_rms(out["tiles"][2], out["rows"][2]) <= 1e-6
