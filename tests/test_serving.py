"""Continuous batching and the job server.

The property under test is the serving contract: a job's result is the same,
bit for bit, whether it runs alone or shares the GPU with jobs that arrive,
finish and fail around it.  The reference has no batched form of this path
(fused_engine.rs:18306, :18433 bail out), so "alone" is one system in its own
batch, stepped in one call.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import pytest


def _alone(pq, topo, params, n_steps):
    b = pq.Batch(max_atoms=topo.n_atoms + 64, max_systems=1)
    s = b.add_system(topo, params)
    b.step(n_steps)
    x, v = b.get_state(s)
    b.close()
    return x, v


def _drain(server, n, timeout_s=240.0):
    out = []
    t_end = time.time() + timeout_s
    while len(out) < n and time.time() < t_end:
        out += server.poll(wait_ms=200)
    assert len(out) == n, f"only {len(out)} of {n} results arrived"
    return {r.job_id: r for r in out}


# ---------------------------------------------------------------- CPU checks
def test_server_structs_match_the_header(pq):
    # sizes of the C structs on LP64 (x86-64 and aarch64): the ctypes mirrors
    # must agree or every field after the first mismatch is misread
    assert ctypes.sizeof(pq.ServerConfigStruct) == 16
    assert ctypes.sizeof(pq.JobStruct) == 136
    assert ctypes.sizeof(pq.ParamsStruct) == 56
    assert ctypes.sizeof(pq.JobResultStruct) == 224
    assert ctypes.sizeof(pq.ServerStatsStruct) == 96


def test_server_without_device_fails_loudly(pq):
    if pq.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(pq.PrismQError) as e:
        pq.Server(1 << 30)
    assert e.value.status == 3  # E_NO_DEVICE


# ---------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def mix(pq):
    """Three chains of different sizes with their own noise streams."""
    return [(pq.Topology.polyala(1, 30, seed=21), pq.Params(stream=101), 120),
            (pq.Topology.polyala(1, 64, seed=22), pq.Params(stream=102), 75),
            (pq.Topology.polyala(1, 110, seed=23), pq.Params(stream=103), 200)]


@pytest.mark.gpu
def test_batch_add_remove_mid_run_matches_alone(gpu, mix):
    (ta, pa, _), (tb, pb, _), (tc, pc, _) = mix
    xa, va = _alone(gpu, ta, pa, 300)
    b = gpu.Batch(max_atoms=ta.n_atoms + tb.n_atoms + tc.n_atoms + 256, max_systems=4)
    sa = b.add_system(ta, pa)
    sb = b.add_system(tb, pb)
    b.step(100)
    b.remove_system(sb)
    sc = b.add_system(tc, pc)  # reuses B's slot and part of its range
    b.step(150)
    sd = b.add_system(tb, gpu.Params(stream=104))
    b.step(50)
    x, v = b.get_state(sa)
    assert b.timestep(sa) == 300 and b.timestep(sc) == 200 and b.timestep(sd) == 50
    assert np.array_equal(x, xa) and np.array_equal(v, va)
    # C joined at step 100 of A's run: its own 200 steps equal C alone
    xc, vc = _alone(gpu, tc, pc, 200)
    xcb, vcb = b.get_state(sc)
    assert np.array_equal(xcb, xc) and np.array_equal(vcb, vc)
    b.close()


@pytest.mark.gpu
def test_served_jobs_match_running_alone(gpu, mix):
    # a long job first; the mix arrives while it is on the GPU
    jobs = [(mix[2][0], gpu.Params(stream=105), 1500)] + list(mix)
    ref = [_alone(gpu, t, p, n) for t, p, n in jobs]
    with gpu.Server(1 << 30, chunk_steps=50) as srv:
        ids = [srv.submit(jobs[0][0], jobs[0][2], jobs[0][1], tag=0)]
        t_end = time.time() + 30
        while srv.stats()["resident_jobs"] == 0 and time.time() < t_end:
            time.sleep(0.001)
        ids += [srv.submit(t, n, p, tag=k) for k, (t, p, n) in enumerate(jobs) if k > 0]
        res = _drain(srv, len(ids))
        st = srv.stats()
    for k, jid in enumerate(ids):
        r = res[jid]
        assert r.ok, r.message
        assert r.tag == k and r.steps_done == jobs[k][2] and r.n_atoms == jobs[k][0].n_atoms
        assert r.submit_s <= r.start_s <= r.end_s
        assert np.array_equal(r.positions, ref[k][0]) and np.array_equal(r.velocities, ref[k][1])
    # the later jobs were admitted while the long one was resident (their work overlapped)
    assert min(res[j].start_s for j in ids[1:]) < res[ids[0]].end_s
    assert st["completed"] == len(jobs) and st["failed"] == 0
    expect = sum(t.n_atoms * n for t, _, n in jobs)
    assert abs(st["atom_steps"] - expect) < 0.5


@pytest.mark.gpu
def test_admission_waits_for_hbm_footprint(gpu, mix):
    big = mix[2][0]
    # an arena that holds one of these jobs but not two
    probe = gpu.Server(1 << 28, max_systems=2)
    per_atom = probe.stats()["device_bytes"] / max(probe.stats()["capacity_atoms"], 1)
    probe.close()
    budget = int(per_atom * (1.5 * big.n_atoms + 64 + 2 * 32))
    ref = _alone(gpu, big, gpu.Params(stream=7), 60)
    with gpu.Server(budget, max_systems=2, chunk_steps=20) as srv:
        cap = srv.stats()["capacity_atoms"]
        assert big.n_atoms <= cap < 2 * big.n_atoms
        ids = [srv.submit(big, 60, gpu.Params(stream=7), tag=i) for i in range(3)]
        res = _drain(srv, 3)
    runs = sorted((res[j].start_s, res[j].end_s) for j in ids)
    for (s0, e0), (s1, e1) in zip(runs, runs[1:]):
        assert s1 >= e0 - 1e-6  # admitted only after the previous job left the arena
    for j in ids:
        assert res[j].ok, res[j].message
        assert np.array_equal(res[j].positions, ref[0]) and np.array_equal(res[j].velocities, ref[1])


@pytest.mark.gpu
def test_oversized_job_rejected_at_submit(gpu, mix):
    with gpu.Server(1 << 26, max_systems=4) as srv:
        cap = srv.stats()["capacity_atoms"]
        huge = gpu.Topology.polyala(1, cap // 10 + 8, seed=5)
        with pytest.raises(gpu.PrismQError) as e:
            srv.submit(huge, 10)
        assert e.value.status == 4  # E_CAPACITY
        jid = srv.submit(mix[0][0], 10, mix[0][1])
        assert _drain(srv, 1)[jid].ok


@pytest.mark.gpu
def test_failing_job_does_not_disturb_the_others(gpu, mix, ala40):
    (ta, pa, na), (tb, pb, nb) = mix[0], mix[1]
    ref_a = _alone(gpu, ta, pa, na)
    ref_b = _alone(gpu, tb, pb, nb)
    bad = gpu.Params(max_constraint_iter=1, temperature=600.0, stream=9)
    with gpu.Server(1 << 30, chunk_steps=25) as srv:
        ia = srv.submit(ta, na, pa)
        ix = srv.submit(ala40, 200, bad)
        ib = srv.submit(tb, nb, pb)
        res = _drain(srv, 3)
    assert res[ix].status in (7, 8) and res[ix].steps_done < 200 and res[ix].message
    for jid, ref in ((ia, ref_a), (ib, ref_b)):
        assert res[jid].ok, res[jid].message
        assert np.array_equal(res[jid].positions, ref[0]) and np.array_equal(res[jid].velocities, ref[1])


@pytest.mark.gpu
def test_served_jobs_follow_their_protocols(gpu, mix):
    """Each job runs its own protocol inside the shared batch, exactly as alone."""
    protos = [gpu.Protocol(start_temp=100.0 + 40 * k, end_temp=300.0, cold_hold_steps=3 * k, ramp_steps=30,
                           warm_hold_steps=20, cryo_enabled=bool(k % 2), equilibration_steps=25,
                           equilibration_gamma=60.0, adaptive_dt=k % 2, current_step=k)
              for k in range(len(mix))]
    ref = []
    for (t, p, n), pr in zip(mix, protos):
        e = gpu.NhsAmberFusedEngine(t, p)
        e.set_protocol(pr)
        e.step(n)
        ref.append((e.get_positions(), e.get_velocities()))
        e.close()
    with gpu.Server(1 << 30, chunk_steps=37) as srv:
        ids = [srv.submit(t, n, p, tag=k, protocol=pr) for k, ((t, p, n), pr) in enumerate(zip(mix, protos))]
        res = _drain(srv, len(ids))
    for k, jid in enumerate(ids):
        r = res[jid]
        assert r.ok, r.message
        assert np.array_equal(r.positions, ref[k][0]) and np.array_equal(r.velocities, ref[k][1])


@pytest.mark.gpu
def test_invalid_protocol_rejected_at_submit(gpu, mix):
    bad = gpu.Protocol(adaptive_dt=5)
    with gpu.Server(1 << 28) as srv:
        with pytest.raises(gpu.PrismQError):
            srv.submit(mix[0][0], 10, mix[0][1], protocol=bad)


@pytest.mark.gpu
def test_job_chain_through_snapshots_equals_one_job(gpu, mix):
    """A 1000-step run split into three served jobs chained by snapshots
    (one of them resumed from an engine's checkpoint) equals the run alone;
    other jobs share the arena meanwhile."""
    t, p, _ = mix[1]
    ref = _alone(gpu, t, p, 1000)
    with gpu.Server(1 << 30, chunk_steps=64) as srv:
        side = srv.submit(mix[0][0], 300, mix[0][1])
        a = srv.submit(t, 400, p, want_snapshot=True)
        res = _drain(srv, 2)
        assert res[a].ok and res[side].ok and res[a].snapshot is not None
        e = gpu.NhsAmberFusedEngine(t, gpu.Params(stream=999))
        e.restore(res[a].snapshot)
        assert e.timestep == 400
        e.step(250)
        b = srv.submit(t, 350, gpu.Params(stream=5), resume=e.checkpoint(), want_snapshot=True)
        rb = _drain(srv, 1)[b]
        e.close()
    assert rb.ok, rb.message
    assert np.array_equal(rb.positions, ref[0]) and np.array_equal(rb.velocities, ref[1])
    f = gpu.NhsAmberFusedEngine(t, gpu.Params())
    f.restore(rb.snapshot)
    assert f.timestep == 1000
    assert np.array_equal(f.get_positions(), ref[0]) and np.array_equal(f.get_velocities(), ref[1])
    f.close()


@pytest.mark.gpu
def test_bad_resume_fails_the_job_alone(gpu, mix, ala40):
    e = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    e.step(3)
    blob = bytearray(e.checkpoint())
    e.close()
    blob[-3] ^= 0x01
    t, p, n = mix[0]
    ref = _alone(gpu, t, p, n)
    with gpu.Server(1 << 30, chunk_steps=40) as srv:
        with pytest.raises(gpu.PrismQError):
            srv.submit(ala40, 10, resume=bytes(blob[:-1]))  # wrong size: refused at submit
        bad = srv.submit(ala40, 10, resume=bytes(blob))
        good = srv.submit(t, n, p)
        res = _drain(srv, 2)
    assert not res[bad].ok and "corrupted" in res[bad].message and res[bad].steps_done == 0
    assert res[good].ok and np.array_equal(res[good].positions, ref[0])


def test_checkpoint_size_for_atoms_is_host_only(pq):
    """Sizing a served job's snapshot buffer needs no device: a fixed header
    plus positions, velocities and list-build positions (9 floats per atom)."""
    L = pq.load()
    sizes = []
    for n in (0, 1, 2500, 100_000):
        out = ctypes.c_size_t()
        assert L.prismq_checkpoint_size_for_atoms(n, ctypes.byref(out)) == 0
        sizes.append(out.value)
    header = sizes[0]
    assert header > 0 and all(s == header + 36 * n for s, n in zip(sizes, (0, 1, 2500, 100_000)))
    assert L.prismq_checkpoint_size_for_atoms(-1, ctypes.byref(ctypes.c_size_t())) == 1


def _dense_cloud(kind):
    rng = np.random.default_rng(3)
    if kind == "rows":  # 8,000 atoms in a 30 Å cube: ≈2,100 partners inside, ≤ 77 atoms per cell
        return (rng.random((8000, 3)) * 30.0).astype(np.float32)
    d = rng.normal(size=(1300, 3))  # 1,300 atoms in a 6 Å ball: three cells, > 512 atoms in one
    d /= np.linalg.norm(d, axis=1)[:, None]
    return (d * 6.0 * rng.random((1300, 1)) ** (1.0 / 3.0)).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,status", [("rows", 6), ("cells", 5)])
def test_list_overflow_is_reported_and_isolated(gpu, kind, status):
    """Clouds dense enough that rows reach the 1024-entry cap
    (PRISMQ_E_NEIGHBOR_OVERFLOW) or a cell the 512-atom cap
    (PRISMQ_E_CELL_OVERFLOW): the writes stop at the caps and the system
    reports the status (no trap).  The system beside it in the same batch is
    untouched and, once the failed one is removed, continues exactly as it
    would alone."""
    dense = gpu.Topology.point_cloud(_dense_cloud(kind))
    ok = gpu.Topology.polyala(1, 20, seed=5)
    b = gpu.Batch(max_atoms=12288, max_systems=4)
    s_ok = b.add_system(ok, gpu.Params(stream=1))
    s_bad = b.add_system(dense, gpu.Params(stream=2))
    with pytest.raises(gpu.PrismQError) as e:
        b.step(5)
    assert e.value.status == status
    assert b.status(s_bad) == status
    assert b.status(s_ok) == 0
    done = b.timestep(s_ok)
    b.remove_system(s_bad)
    b.step(7)
    x, v = b.get_state(s_ok)
    b.close()
    xr, vr = _alone(gpu, ok, gpu.Params(stream=1), done + 7)
    assert np.array_equal(x, xr) and np.array_equal(v, vr)
