"""Run protocol: per-step temperature, friction and timestep (ProtocolState +
director, protocol_state.cuh:14-62, protocol_director.cu:54-143; friction
compute_cryo_friction, fused_engine.rs:15366-15396).

Bars: the library's director values equal the oracle's C restatement bit for
bit and the reference formulas (restated here in numpy float32) to the last
bit; on the GPU every protocol step equals the oracle's reference phase order
fed the device forces, bit for bit, with the protocol evaluated inside the
captured step graph.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

F = np.float32


def _protocols(pq):
    return [
        pq.Protocol(),
        pq.Protocol(start_temp=50.0, end_temp=300.0, cold_hold_steps=3, ramp_steps=7, warm_hold_steps=5,
                    ramp_down_steps=4, cold_return_steps=2, cryo_enabled=True, equilibration_steps=12,
                    adaptive_dt=1),
        pq.Protocol(start_temp=100.0, end_temp=310.0, ramp_steps=11, warm_hold_steps=0, adaptive_dt=2,
                    equilibration_steps=0, gamma_base=0.0),
        pq.Protocol(start_temp=5.0, end_temp=280.0, cold_hold_steps=1, ramp_steps=1, warm_hold_steps=1,
                    ramp_down_steps=1, cold_return_steps=0, cryo_enabled=True, equilibration_steps=3,
                    equilibration_gamma=250.0, gamma_base=2.5, base_dt=0.002, current_step=7),
    ]


def _numpy_director(p, s):
    """prism_protocol_baseline_v1 in numpy float32 (protocol_director.cu:54-143)."""
    e1 = p.cold_hold_steps
    e2 = e1 + p.ramp_steps
    e3 = e2 + p.warm_hold_steps
    e4 = e3 + p.ramp_down_steps
    st, et = F(p.start_temp), F(p.end_temp)
    if s < e1:
        T, hold = st, True
    elif s < e2:
        T, hold = st + (F(s - e1) / F(e2 - e1)) * (et - st), False
    elif s < e3:
        T, hold = et, True
    elif s < e4:
        T, hold = et - (F(s - e3) / F(e4 - e3)) * (et - st), False
    else:
        T, hold = (et if p.ramp_down_steps == 0 and p.cold_return_steps == 0 else st), True
    g = F(p.gamma_base)
    if s < p.equilibration_steps:
        decay = F(np.exp(np.float64(F(-3.0) * (F(s) / F(p.equilibration_steps)))))
        g = F(p.equilibration_gamma) * decay + F(p.gamma_base) * (F(1.0) - decay)
    if p.cryo_enabled and T < F(300.0):
        g = g * np.sqrt(F(300.0) / max(T, F(10.0)))
    dt = F(p.base_dt)
    if p.adaptive_dt == 2:
        dt = dt * F(1.5) if hold else dt
    elif p.adaptive_dt == 1:
        dt = dt if hold else dt * F(0.5)
    return float(F(T)), float(F(g)), float(F(dt))


STEPS = list(range(0, 40)) + [9998, 9999, 10000, 10001, 123456, 2 ** 31 - 1]


def test_director_matches_oracle_restatement(pq, orc):
    for p in _protocols(pq):
        ps = p.struct()
        for s in STEPS:
            assert p.eval(s) == orc.protocol_eval(ps, s)[:3], (p, s)


def test_director_matches_reference_formulas(pq):
    for p in _protocols(pq):
        for s in STEPS:
            assert p.eval(s) == _numpy_director(p, s), (p, s)


def test_director_known_points(pq):
    p = pq.Protocol(start_temp=50.0, end_temp=300.0, cold_hold_steps=10, ramp_steps=10, warm_hold_steps=10,
                    cryo_enabled=True, adaptive_dt=1)
    assert p.eval(0) == (50.0, float(F(1000.0) * np.sqrt(F(6.0))), float(F(0.004)))  # decay e^0 = 1
    assert p.eval(15)[0] == 175.0 and p.eval(15)[2] == float(F(0.002))                # mid-ramp, half dt
    assert p.eval(25)[0] == 300.0 and p.eval(10000)[1] == 1.0                           # warm hold, γ settled
    assert p.eval(10 ** 6)[0] == 300.0                                                   # warm tail (no cooling)
    q = pq.Protocol(start_temp=50.0, end_temp=300.0, warm_hold_steps=1, ramp_down_steps=1, cold_return_steps=1)
    assert q.eval(5)[0] == 50.0                                                          # cold return


@pytest.mark.parametrize("field,value", [("ramp_steps", -1), ("adaptive_dt", 3), ("base_dt", 0.0),
                                         ("start_temp", float("nan")), ("gamma_base", -1.0),
                                         ("current_step", -2), ("cryo_enabled", 2)])
def test_invalid_protocol_refused(pq, field, value):
    ps = pq.Protocol().struct()
    setattr(ps, field, value)
    out = (ctypes.c_float * 3)()
    assert pq.load().prismq_protocol_eval(ctypes.byref(ps), 1, out) == 1


def test_protocol_struct_layout(pq):
    assert ctypes.sizeof(pq.ProtocolStruct) == 56
    L = pq.load()
    d = pq.ProtocolStruct()
    L.prismq_protocol_default(ctypes.byref(d))
    want = pq.Protocol().struct()
    assert bytes(d) == bytes(want)


# ---------------------------------------------------------------- GPU
def _oracle_sys(orc, topo, p):
    return orc.OracleSystem(topo.struct(), dt=p.dt, temperature=p.temperature, gamma=p.gamma, cutoff=p.cutoff,
                            max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed,
                            stream=p.stream)


def _ramp(pq, **kw):
    base = dict(start_temp=120.0, end_temp=300.0, cold_hold_steps=2, ramp_steps=5, warm_hold_steps=3,
                ramp_down_steps=4, cold_return_steps=2, cryo_enabled=True, equilibration_steps=9,
                equilibration_gamma=40.0, gamma_base=1.0, adaptive_dt=1, base_dt=0.004)
    base.update(kw)
    return pq.Protocol(**base)


@pytest.mark.gpu
@pytest.mark.parametrize("start_step", [0, 95])
def test_protocol_steps_bit_exact(gpu, orc, ala40, start_step):
    """Every step of a protocol (ramps, holds, friction blend, cryo scaling,
    adaptive dt; start 95 crosses the COM removal at step 100) equals the
    oracle's phases with the director's values for that step, fed the device
    forces."""
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    eng.step(2)
    eng.set_timestep(start_step)
    proto = _ramp(gpu)
    eng.set_protocol(proto)
    o = _oracle_sys(orc, ala40, p)
    o.set_protocol(proto.struct(), start_step - (proto.current_step + 1))
    for k in range(18):
        st = start_step + k
        want = orc.protocol_eval(proto.struct(), k + 1)
        assert eng.step_params() == want[:3], k
        x, v = eng.get_positions(), eng.get_velocities()
        _, _, f_n = eng.compute_forces()
        eng.step(1)
        _, _, f_np1 = eng.compute_forces()
        o.set_state(x, v)
        if st > 0 and st % p.com_interval == 0:
            o.com_remove()
        assert o.phases(1, f_n, st) == 0
        assert o.phases(2, f_np1, st) == 0
        xo, vo = o.get_state()
        assert np.array_equal(eng.get_positions(), xo), k
        assert np.array_equal(eng.get_velocities(), vo), k
    eng.close()


@pytest.mark.gpu
def test_protocol_in_graph_equals_single_steps(gpu, ala40):
    """The director runs inside the captured graph: 30 steps in one call equal
    30 calls of one step."""
    proto = _ramp(gpu, ramp_steps=9, warm_hold_steps=6)
    a = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    b = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    a.set_protocol(proto)
    b.set_protocol(proto)
    a.step(30)
    for _ in range(30):
        b.step(1)
    assert np.array_equal(a.get_positions(), b.get_positions())
    assert np.array_equal(a.get_velocities(), b.get_velocities())
    assert a.step_params() == b.step_params() == proto.eval(31)
    a.close()
    b.close()


@pytest.mark.gpu
def test_protocol_per_system_in_a_batch(gpu):
    """Systems of one batch follow their own protocols, and each equals its solo run."""
    topos = [gpu.Topology.polyala(1, 12, seed=3), gpu.Topology.polyala(1, 20, seed=4)]
    protos = [_ramp(gpu), _ramp(gpu, start_temp=200.0, adaptive_dt=2, cryo_enabled=False, current_step=3)]
    bat = gpu.Batch(max_atoms=1024, max_systems=4)
    slots = [bat.add_system(t, gpu.Params(stream=i)) for i, t in enumerate(topos)]
    for s, pr in zip(slots, protos):
        bat.set_protocol(s, pr)
    bat.step(25)
    for i, (t, pr) in enumerate(zip(topos, protos)):
        e = gpu.NhsAmberFusedEngine(t, gpu.Params(stream=i))
        e.set_protocol(pr)
        e.step(25)
        x, v = bat.get_state(slots[i])
        assert np.array_equal(x, e.get_positions()) and np.array_equal(v, e.get_velocities())
        assert bat.step_params(slots[i]) == e.step_params() == pr.eval(pr.current_step + 26)
        e.close()
    bat.close()


@pytest.mark.gpu
def test_protocol_setter_rules(gpu, ala40):
    eng = gpu.NhsAmberFusedEngine(ala40, gpu.Params())
    proto = _ramp(gpu)
    eng.set_protocol(proto)
    with pytest.raises(gpu.PrismQError):
        eng.set_temperature(250.0)
    with pytest.raises(gpu.PrismQError):
        eng.set_gamma(2.0)
    eng.set_dt(0.003)  # moves base_dt (set_dt, fused_engine.rs:15342)
    proto.base_dt = 0.003
    assert eng.step_params() == proto.eval(1)
    eng.step(5)
    params = eng.step_params()
    assert params == proto.eval(6)
    eng.set_protocol(None)  # the system keeps the values it had
    assert eng.step_params() == params
    eng.step(3)
    assert eng.step_params() == params
    eng.set_temperature(250.0)
    assert eng.step_params()[0] == 250.0
    eng.close()


@pytest.mark.gpu
def test_parameter_change_applies_to_the_whole_next_step(gpu, orc, ala40):
    """Without a protocol, a temperature / friction change between calls
    governs both halves of the next step, as in the reference's step()."""
    p = gpu.Params()
    eng = gpu.NhsAmberFusedEngine(ala40, p)
    eng.step(4)
    x, v = eng.get_positions(), eng.get_velocities()
    _, _, f_n = eng.compute_forces()
    eng.set_temperature(150.0)
    eng.set_gamma(5.0)
    eng.step(1)
    _, _, f_np1 = eng.compute_forces()
    o = orc.OracleSystem(ala40.struct(), dt=p.dt, temperature=150.0, gamma=5.0, cutoff=p.cutoff,
                         max_iter=p.max_constraint_iter, com_interval=p.com_interval, seed=p.seed,
                         stream=p.stream)
    o.set_state(x, v)
    assert o.phases(1, f_n, 4) == 0 and o.phases(2, f_np1, 4) == 0
    xo, vo = o.get_state()
    assert np.array_equal(eng.get_positions(), xo) and np.array_equal(eng.get_velocities(), vo)
    eng.close()
