"""Whole-arena state transfer (prismq_batch_set_state_all / get_state_all).

Pinned host arrays are read and written by the transfer kernel directly over
the host link; pageable arrays go through a device staging copy.  Bar: every
form gives the per-system states bit for bit, including an arena span whose
last 256-atom block is partial and pinned arrays that are not 16-byte aligned
(the kernel then moves single words instead of 16-byte vectors), and a
whole-arena upload continues exactly as the same upload per system.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(n, offset_floats=0):
    torch = pytest.importorskip("torch")
    t = torch.empty(n + offset_floats, dtype=torch.float32, pin_memory=True)
    return t, t.numpy()[offset_floats:]  # the tensor keeps the pinned block alive


def _batch(gpu, topos):
    b = gpu.Batch(max_atoms=4096, max_systems=4)
    slots = [b.add_system(t, gpu.Params(stream=k)) for k, t in enumerate(topos)]
    b.step(12)
    return b, slots


@pytest.fixture(scope="module")
def topos(gpu):
    return [gpu.Topology.polyala(1, n, seed=50 + n) for n in (7, 45, 130)]


def _views(b, s, n, x, v):
    o = b.atom_offset(s)
    return x[3 * o:3 * (o + n)].reshape(-1, 3), v[3 * o:3 * (o + n)].reshape(-1, 3)


@pytest.mark.parametrize("form", ["pageable", "pinned", "pinned_misaligned"])
def test_get_state_all_matches_each_system(gpu, topos, form):
    b, slots = _batch(gpu, topos)
    span = b.atom_span()
    assert span % 256 != 0  # the last transfer block is partial
    keep = []
    if form == "pageable":
        x, v = b.get_state_all()
    else:
        off = 1 if form == "pinned_misaligned" else 0
        tx, x = _pinned(3 * span, off)
        tv, v = _pinned(3 * span, off)
        keep += [tx, tv]
        x[:] = np.nan
        v[:] = np.nan
        b.get_state_all(x, v)
    for s, t in zip(slots, topos):
        want = b.get_state(s)
        got = _views(b, s, t.n_atoms, x, v)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    b.close()


@pytest.mark.parametrize("form", ["pageable", "pinned", "pinned_misaligned"])
def test_set_state_all_equals_per_system_upload(gpu, topos, form):
    a, slots = _batch(gpu, topos)
    ref, rslots = _batch(gpu, topos)
    span = a.atom_span()
    x, v = a.get_state_all()
    x2 = x.copy()
    v2 = (v * np.float32(0.5)).astype(np.float32)
    o = a.atom_offset(slots[1])
    x2[3 * o:3 * o + 3] += np.float32(0.01)  # one moved atom: that system refreshes its list and forces
    keep = []
    if form != "pageable":
        off = 1 if form == "pinned_misaligned" else 0
        tx, px = _pinned(3 * span, off)
        tv, pv = _pinned(3 * span, off)
        keep += [tx, tv]
        px[:] = x2
        pv[:] = v2
        x2, v2 = px, pv
    a.set_state_all(x2, v2)
    # per system: velocities everywhere, positions only where bits changed
    # (the whole-arena upload refreshes only the systems whose positions moved)
    for k, (s, t) in enumerate(zip(rslots, topos)):
        xs, vs = _views(a, slots[k], t.n_atoms, np.array(x2), np.array(v2))
        ref.set_state(s, xs if k == 1 else None, vs)
    a.step(15)
    ref.step(15)
    for s, rs in zip(slots, rslots):
        xa, va = a.get_state(s)
        xr, vr = ref.get_state(rs)
        assert np.array_equal(xa, xr) and np.array_equal(va, vr)
    a.close()
    ref.close()


@pytest.mark.parametrize("form", ["pageable", "pinned"])
def test_step_host_equals_upload_step_download(gpu, topos, form):
    """prismq_batch_step_host (upload, steps, read-back, one wait) gives the
    same bits as the three calls, in place (the same arrays in and out) or
    not, and with n_steps 0 it only transfers."""
    a, _ = _batch(gpu, topos)
    b, _ = _batch(gpu, topos)
    span = a.atom_span()
    x, v = a.get_state_all()
    v = (v * np.float32(0.9)).astype(np.float32)
    keep = []
    if form == "pinned":
        tx, px = _pinned(3 * span)
        tv, pv = _pinned(3 * span)
        keep += [tx, tv]
        px[:] = x
        pv[:] = v
        x, v = px, pv
    xr, vr = x.copy(), v.copy()
    for _ in range(3):
        a.step_host(4, x, v, x, v)  # in place
        b.set_state_all(xr, vr)
        b.step(4)
        b.get_state_all(xr, vr)
        assert np.array_equal(x, xr) and np.array_equal(v, vr)
    xo, vo = np.empty_like(xr), np.empty_like(vr)
    a.step_host(0, None, None, xo, vo)
    assert np.array_equal(xo, xr) and np.array_equal(vo, vr)
    a.close()
    b.close()


def test_step_host_read_back_on_com_steps(gpu, topos):
    """The pinned read-back of step_host takes the positions while the last
    step's forces run; on a COM step the deferred pre-force phases move the
    positions inside the control kernel, so those calls must still return the
    final positions (COM removal every second step, calls of 1-3 steps)."""
    def batch():
        b = gpu.Batch(max_atoms=4096, max_systems=4)
        for k, t in enumerate(topos):
            b.add_system(t, gpu.Params(stream=k, com_interval=2))
        b.step(5)
        return b

    a, b = batch(), batch()
    span = a.atom_span()
    x, v = a.get_state_all()
    tx, px = _pinned(3 * span)
    tv, pv = _pinned(3 * span)
    px[:] = x
    pv[:] = v
    xr, vr = x.copy(), v.copy()
    for n in (1, 2, 3, 1, 1, 2):
        a.step_host(n, px, pv, px, pv)
        b.set_state_all(xr, vr)
        b.step(n)
        b.get_state_all(xr, vr)
        assert np.array_equal(px, xr) and np.array_equal(pv, vr)
    del tx, tv
    a.close()
    b.close()
