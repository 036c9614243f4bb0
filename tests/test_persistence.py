"""State persistence: checkpoints (capture / restore of the MD state,
fused_engine.rs:24718-25772) and trajectory frames.

Bars: a system restored from a checkpoint continues bit for bit as the saved
one (positions, velocities, forces, step counter, protocol values), in a
fresh system or in a batch slot; damaged or foreign checkpoints are refused;
recorded frames equal the states the engine reports at the same step
boundaries, and recording them changes nothing.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_state(a, b):
    return np.array_equal(a.get_positions(), b.get_positions()) and np.array_equal(
        a.get_velocities(), b.get_velocities())


@pytest.mark.parametrize("split", [0, 1, 20, 33])
def test_checkpoint_resume_bit_exact(gpu, ala40, split):
    """Split 0 saves before the first list build, 20 at a rebuild step, 33
    between rebuilds (13 steps into the list's interval)."""
    total = 60
    a = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    a.step(total)
    b = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    b.step(split)
    blob = b.checkpoint()
    b.close()
    c = gpu.NhsAmberFusedEngine(ala40, gpu.Params(seed=12345, temperature=200.0))  # params come from the blob
    c.restore(blob)
    assert c.timestep == split
    c.step(total - split)
    assert c.timestep == total
    assert _same_state(a, c)
    assert np.array_equal(a.compute_forces()[2], c.compute_forces()[2])
    a.close()
    c.close()


def test_checkpoint_carries_the_protocol(gpu, ala40):
    proto = gpu.Protocol(start_temp=150.0, end_temp=300.0, cold_hold_steps=5, ramp_steps=20, warm_hold_steps=10,
                         cryo_enabled=True, equilibration_steps=30, equilibration_gamma=50.0, adaptive_dt=1)
    a = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    a.set_protocol(proto)
    a.step(40)
    b = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    b.set_protocol(proto)
    b.step(17)
    blob = b.checkpoint()
    c = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    c.restore(blob)
    assert c.step_params() == b.step_params() == proto.eval(18)
    c.step(23)
    assert _same_state(a, c)
    assert c.step_params() == a.step_params()
    for e in (a, b, c):
        e.close()


def test_checkpoint_moves_between_engine_and_batch(gpu, ala40):
    solo = gpu.NhsAmberFusedEngine(ala40, gpu.Params(stream=3))
    solo.step(50)
    src = gpu.NhsAmberFusedEngine(ala40, gpu.Params(stream=3))
    src.step(25)
    blob = src.checkpoint()
    others = [gpu.Topology.polyala(1, 15, seed=8), gpu.Topology.polyala(1, 9, seed=9)]
    bat = gpu.Batch(max_atoms=4096, max_systems=4)
    s0 = bat.add_system(others[0], gpu.Params(stream=1))
    s1 = bat.add_system(ala40, gpu.Params(stream=99))
    s2 = bat.add_system(others[1], gpu.Params(stream=2))
    bat.restore(s1, blob)
    bat.step(25)
    x, v = bat.get_state(s1)
    assert np.array_equal(x, solo.get_positions()) and np.array_equal(v, solo.get_velocities())
    for slot, topo, stream in ((s0, others[0], 1), (s2, others[1], 2)):  # neighbours unaffected
        e = gpu.NhsAmberFusedEngine(topo, gpu.Params(stream=stream))
        e.step(25)
        x, v = bat.get_state(slot)
        assert np.array_equal(x, e.get_positions()) and np.array_equal(v, e.get_velocities())
        e.close()
    back = bat.checkpoint(s1)  # and from the batch into a single system
    d = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    d.restore(back)
    d.step(5)
    solo.step(5)
    assert _same_state(d, solo)
    for e in (solo, src, d):
        e.close()
    bat.close()


def test_checkpoint_refusals(gpu, ala40, tmp_path):
    e = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    e.step(5)
    blob = e.checkpoint()
    # another conformation of the same topology is the same system: accepted
    same = gpu.NhsAmberFusedEngine(gpu.Topology.polyala(1, 40, seed=12), gpu.Params())
    same.restore(blob)
    assert np.array_equal(same.get_positions(), e.get_positions())
    same.close()
    # one changed charge makes another topology
    t2 = gpu.Topology.polyala(1, 40, seed=11)
    t2.charges[5] += np.float32(0.01)
    other = gpu.NhsAmberFusedEngine(t2, gpu.Params())
    with pytest.raises(gpu.PrismQError, match="another topology"):
        other.restore(blob)
    small = gpu.NhsAmberFusedEngine(gpu.Topology.polyala(1, 39, seed=11), gpu.Params())
    with pytest.raises(gpu.PrismQError, match="another size"):
        small.restore(blob)
    small.close()
    bad = bytearray(blob)
    bad[len(bad) - 5] ^= 0x10
    with pytest.raises(gpu.PrismQError, match="corrupted"):
        e.restore(bytes(bad))
    with pytest.raises(gpu.PrismQError):
        e.restore(blob[:-4])
    with pytest.raises(gpu.PrismQError):
        e.restore(b"XXXXXXXX" + blob[8:])
    x_before = e.get_positions()
    assert np.array_equal(e.get_positions(), x_before)  # a refused restore leaves the system as it was
    path = tmp_path / "sys.ckpt"
    e.save_checkpoint(path)
    e.step(7)
    e.load_checkpoint(path)
    assert e.timestep == 5 and np.array_equal(e.get_positions(), x_before)
    f64 = gpu.NhsAmberFusedEngine(ala40, gpu.Params(precision=gpu.PRECISION_FP64))
    with pytest.raises(gpu.PrismQError, match="FP32"):
        f64.checkpoint()
    for s in (e, other, f64):
        s.close()


def test_frames_equal_reported_states(gpu, ala40):
    rec = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    rec.record_frames(7, capacity=32, velocities=True)
    ref = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    rec.step(40)
    rec.step(30)
    want_x, want_v = [], []
    for _ in range(10):
        ref.step(7)
        want_x.append(ref.get_positions())
        want_v.append(ref.get_velocities())
    fr = rec.read_frames()
    assert fr["steps"].tolist() == list(range(7, 71, 7)) and fr["dropped"] == 0
    assert np.array_equal(fr["positions"], np.stack(want_x))
    assert np.array_equal(fr["velocities"], np.stack(want_v))
    assert _same_state(rec, ref)  # recording does not perturb the run
    assert rec.read_frames()["steps"].size == 0  # frames are handed out once
    rec.close()
    ref.close()


def test_frames_ring_keeps_the_newest(gpu, ala40):
    e = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    e.record_frames(2, capacity=3)
    e.step(20)
    fr = e.read_frames()
    assert fr["steps"].tolist() == [16, 18, 20] and fr["dropped"] == 7
    assert fr["velocities"] is None
    np.testing.assert_array_equal(fr["positions"][-1], e.get_positions())
    e.record_frames(0)
    with pytest.raises(gpu.PrismQError):
        e.read_frames()
    e.close()


def test_frames_per_system_in_a_batch(gpu):
    topos = [gpu.Topology.polyala(1, 12, seed=3), gpu.Topology.polyala(1, 20, seed=4)]
    bat = gpu.Batch(max_atoms=2048, max_systems=4)
    slots = [bat.add_system(t, gpu.Params(stream=i)) for i, t in enumerate(topos)]
    bat.record_frames(slots[0], 3, capacity=16)
    bat.record_frames(slots[1], 5, capacity=16, velocities=True)
    bat.step(30)
    for i, (t, interval) in enumerate(zip(topos, (3, 5))):
        fr = bat.read_frames(slots[i], t.n_atoms)
        assert fr["steps"].tolist() == list(range(interval, 31, interval))
        e = gpu.NhsAmberFusedEngine(t, gpu.Params(stream=i))
        for k, st in enumerate(fr["steps"]):
            e.step(int(st) - e.timestep)
            assert np.array_equal(fr["positions"][k], e.get_positions())
            if interval == 5:
                assert np.array_equal(fr["velocities"][k], e.get_velocities())
        e.close()
    bat.close()
