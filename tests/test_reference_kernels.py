"""Pins of the CPU oracle against the reference's OWN device code.

oracle/build_ref.py compiles the reference's nhs_amber_fused.cu (from the
reference tree, here, at build time) into device-only cubins together with
thin wrappers (oracle/ref_harness.cu); oracle/ref_kernels.py runs them on the
GPU.  The same inputs go through the oracle's restatement:

  * integrator pieces — half-kick (clamped and Hamiltonian), RATTLE, SHAKE and
    the velocity clamp kernel — bit-exact against the reference functions
    built without FMA contraction (the oracle's arithmetic), so every phase
    of the restatement performs the reference's operations in its order;
  * force laws, per term — bonds bit-exact (IEEE operations only); angles and
    torsions within 1e-4 of the RMS force of their kind (worst element,
    measured ~3e-5: the reference uses CUDA's acosf/asinf/sinf, the oracle the
    C library's); ordinary pairs and exact 1-4 exceptions within 1e-5 of their
    LJ + Coulomb magnitude against an FP64 statement of the law (the
    reference uses rsqrtf);
  * whole-system forces summed from the reference's per-term functions
    against the oracle's FP32 gather and the production kernels: relative
    RMS <= 1e-5; energies within 1e-6.

Inputs are validated on the host first (indices in range, constraint
clusters that the oracle converges), so no reference failure path runs.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref, ref_kernels

    build_ref.build()
    if not ref_kernels.available():
        pytest.skip("oracle/_ref cubins are not built (the reference tree is needed to build them)")
    return ref_kernels


@pytest.fixture(scope="module")
def sysx(pq):
    """A 100-residue chain at positions displaced from the grown geometry, so
    every term carries force."""
    topo = pq.Topology.polyala(1, 100, seed=31)
    rng = np.random.default_rng(5)
    x = (topo.positions + rng.normal(0.0, 0.04, topo.positions.shape)).astype(np.float32)
    return topo, x


def _orc(orc, topo, gamma=1.0, dt=0.004, temperature=300.0):
    return orc.OracleSystem(topo.struct(), dt=dt, gamma=gamma, temperature=temperature)


def _pairs(topo, x, r_max=10.5):
    """Ordinary pairs (not excluded) within r_max and the exact exceptions."""
    from scipy.spatial import cKDTree

    n = topo.n_atoms
    excl = set()
    off, lst = topo.exclusion_offsets, topo.exclusions
    for i in range(n):
        for j in lst[off[i]:off[i + 1]]:
            excl.add((min(i, int(j)), max(i, int(j))))
    cand = cKDTree(x.astype(np.float64)).query_pairs(r_max, output_type="ndarray")
    ordinary = np.array([p for p in map(tuple, cand.tolist()) if (min(p), max(p)) not in excl], np.int32)
    ex = topo.exceptions
    exc = np.stack([ex["i"], ex["j"]], 1).astype(np.int32)
    pairs = np.concatenate([ordinary.reshape(-1, 2), exc])
    exact = np.concatenate([np.zeros(len(ordinary), np.int32), np.ones(len(exc), np.int32)])
    params = np.zeros((len(pairs), 3), np.float32)
    params[len(ordinary):] = np.stack([ex["charge_product"], ex["sigma"], ex["epsilon"]], 1)
    return pairs, exact, params


def _accumulate(n, idx, f):
    out = np.zeros((n, 3), np.float64)
    for m in range(idx.shape[1]):
        np.add.at(out, idx[:, m], f[:, m].astype(np.float64))
    return out


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return int(np.abs(a - b).max()) if a.size else 0


# ---------------------------------------------------------------- force laws
def test_bonded_terms_match_reference_functions(pq, orc, ref, sysx):
    topo, x = sysx
    o = _orc(orc, topo)
    o.set_state(x, np.zeros_like(x))
    fb, fa, fd = o.term_forces(len(topo.bonds), len(topo.angles), len(topo.dihedrals))
    o.close()
    # bonds: IEEE operations only -> identical bits without contraction
    rb, _ = ref.bond_terms(topo, x, nofma=True)
    assert np.array_equal(rb, fb)
    # angles and torsions: CUDA vs C-library acos/asin/sin differ by a few ulp;
    # errors are measured against the RMS force of the term kind (a torsion
    # near a zero of sin(n phi - gamma) has a tiny force with an ulp-sized error)
    worst = {}
    for name, got, want in (("angle", ref.angle_terms(topo, x, nofma=True)[0], fa),
                            ("torsion", ref.dihedral_terms(topo, x, nofma=True)[0], fd),
                            ("bond/fma", ref.bond_terms(topo, x)[0], fb),
                            ("angle/fma", ref.angle_terms(topo, x)[0], fa),
                            ("torsion/fma", ref.dihedral_terms(topo, x)[0], fd)):
        rms = np.sqrt((want.astype(np.float64) ** 2).mean()) + 1e-30
        worst[name] = float(np.abs(got.astype(np.float64) - want).max() / rms)
    assert max(worst.values()) <= 1e-4, worst


def test_pair_law_matches_reference_function(pq, orc, ref, sysx):
    topo, x = sysx
    pairs, exact, params = _pairs(topo, x)
    rf, rpe = ref.pair_terms(topo, x, pairs, exact, params)
    # restate the pair law in FP64 from the same inputs: LJ (Lorentz-Berthelot)
    # + Coulomb 332.0636 q q / r, exceptions with their own (qq, sigma, eps);
    # ordinary pairs beyond the cutoff contribute nothing
    d = x[pairs[:, 1]].astype(np.float64) - x[pairs[:, 0]]
    r2 = (d ** 2).sum(1)
    q, s, e = topo.charges.astype(np.float64), topo.lj_sigma.astype(np.float64), topo.lj_epsilon.astype(np.float64)
    sig = np.where(exact == 1, params[:, 1], 0.5 * (s[pairs[:, 0]] + s[pairs[:, 1]]))
    eps = np.where(exact == 1, params[:, 2], np.sqrt(e[pairs[:, 0]] * e[pairs[:, 1]]))
    qq = np.where(exact == 1, params[:, 0], q[pairs[:, 0]] * q[pairs[:, 1]])
    sr6 = (sig ** 2 / r2) ** 3
    f_lj = 24.0 * eps / r2 * (2.0 * sr6 * sr6 - sr6)
    f_c = 332.0636 * qq / r2 / np.sqrt(r2)
    live = (exact == 1) | (r2 <= 100.0)
    fs = np.where(live, f_lj + f_c, 0.0)
    want_i = -fs[:, None] * d
    # FP32 rounding is relative to the LJ and Coulomb parts, which can cancel
    scale = np.where(live, np.abs(f_lj) + np.abs(f_c), 0.0) * np.sqrt(r2) + 1e-6
    err = np.abs(rf[:, 0] - want_i).max(1) / scale
    assert err.max() <= 1e-5, (float(err.max()), int(err.argmax()))
    assert np.array_equal(rf[:, 0], -rf[:, 1])
    # the reference's per-atom halves sum to the pair energy (shifted for ordinary pairs)
    assert np.all(np.isfinite(rpe))


def test_system_forces_and_energy_match_reference_functions(pq, orc, ref, sysx, gpu):
    topo, x = sysx
    n = topo.n_atoms
    b = topo.bonds
    a = topo.angles
    t = topo.dihedrals
    rb, pb = ref.bond_terms(topo, x)
    ra, pa = ref.angle_terms(topo, x)
    rd, pd = ref.dihedral_terms(topo, x)
    pairs, exact, params = _pairs(topo, x)
    rp, pp = ref.pair_terms(topo, x, pairs, exact, params)
    f_ref = (_accumulate(n, np.stack([b["i"], b["j"]], 1), rb) +
             _accumulate(n, np.stack([a["i"], a["j"], a["k"]], 1), ra) +
             _accumulate(n, np.stack([t["i"], t["j"], t["k"], t["l"]], 1), rd) +
             _accumulate(n, pairs, rp))
    e_ref = np.array([pb.sum(), pa.sum(), pd.sum(), pp[exact == 1].sum(), pp[exact == 0].sum()])
    # the oracle's FP32 gather (REF27 rows) and its FP64 forces
    o = _orc(orc, topo)
    o.set_state(x, np.zeros_like(x))
    f32, e32 = o.forces_ref_f32()
    f64, e64 = o.forces_f64()
    o.close()
    assert rel_rms(f32, f_ref) <= 1e-5
    assert rel_rms(f64, f_ref) <= 1e-5
    for k in range(5):
        assert abs(e64[k] - e_ref[k]) <= 1e-6 * max(abs(e_ref[k]), 1.0), (k, e64[k], e_ref[k])
    # the production kernels at the same positions
    eng = gpu.NhsAmberFusedEngine(gpu.Topology(x, topo.masses, topo.charges, topo.lj_sigma, topo.lj_epsilon,
                                               topo.bonds, topo.angles, topo.dihedrals, topo.exceptions,
                                               topo.exclusion_offsets, topo.exclusions, topo.clusters),
                                  gpu.Params())
    pe, f, _ = eng.compute_forces()
    comp = eng.energy_components()
    eng.close()
    assert rel_rms(f, f_ref) <= 1e-5
    for k in range(5):
        assert abs(comp[k] - e_ref[k]) <= 1e-6 * max(abs(e_ref[k]), 1.0), (k, comp[k], e_ref[k])


# ---------------------------------------------------------------- integrator
def _thermal(topo, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    sd = np.sqrt(418.4 * 0.001987204 * 300.0 / topo.masses.astype(np.float64))[:, None]
    return (rng.normal(0.0, 1.0, (topo.n_atoms, 3)) * sd * scale).astype(np.float32)


@pytest.mark.parametrize("gamma", [1.0, 0.0])
def test_half_kick_bit_exact_with_reference(pq, orc, ref, sysx, gamma):
    topo, x = sysx
    v = _thermal(topo, 1)
    rng = np.random.default_rng(2)
    f = (rng.normal(0.0, 300.0, v.shape)).astype(np.float32)  # some |F| above the 1000 clamp
    f[::7] *= 8.0
    o = _orc(orc, topo, gamma=gamma)
    o.set_state(x, v)
    o.kick_all(f)
    _, v_orc = o.get_state()
    o.close()
    v_ref = ref.kick(v, f, topo.masses, 0.004, exact=(gamma == 0.0))
    assert np.array_equal(v_ref, v_orc)


@pytest.mark.parametrize("gamma,dt,temperature", [(1.0, 0.004, 300.0), (5.0, 0.002, 250.0), (1000.0, 0.004, 300.0)])
def test_ou_half_step_bit_exact_with_reference(pq, orc, ref, sysx, gamma, dt, temperature):
    """The OU half-step (langevin_thermostat as the OU phases call it) from
    the reference's own cuRAND draws: given the normals it drew and its c1,
    the oracle's OU update, which the production integrator reproduces bit
    for bit with its own (Philox) normals, equals the reference's.  The
    library's c1, exp(-γ dt/2) in binary64 rounded to float, is within one
    float ulp of the device expf the reference evaluates."""
    topo, x = sysx
    v = _thermal(topo, 7)
    v_ref, z, c1_ref = ref.ou(v, topo.masses, temperature, gamma, dt, seed=0x5052_4953_4d5f_4d42)
    assert np.isfinite(z).all() and 0.5 < float(np.std(z)) < 1.5  # the draws are standard normals
    o = _orc(orc, topo, gamma=gamma, dt=dt, temperature=temperature)
    o.set_state(x, v)
    o.ou_all(z, c1_ref)
    _, v_orc = o.get_state()
    o.close()
    assert np.array_equal(v_ref, v_orc)
    c1_lib = np.float32(orc.c1_of(gamma, dt))
    assert abs(int(c1_lib.view(np.int32)) - int(np.float32(c1_ref).view(np.int32))) <= 1
    # with the reference's own compiler flags (FMA contraction on) cuRAND's
    # normals and the update differ from the uncontracted build by rounding only
    v_fma, z2, _ = ref.ou(v, topo.masses, temperature, gamma, dt, seed=0x5052_4953_4d5f_4d42, nofma=False)
    assert rel_rms(z2, z) <= 1e-6
    assert rel_rms(v_fma, v_ref) <= 1e-6


def test_rattle_bit_exact_with_reference(pq, orc, ref, sysx):
    topo, _ = sysx
    x = topo.positions  # constrained geometry
    v = _thermal(topo, 3)
    o = _orc(orc, topo)
    o.set_state(x, v)
    assert o.rattle_all() == 0  # converges on the CPU first
    _, v_orc = o.get_state()
    o.close()
    v_ref, ok = ref.rattle(topo, x, v)
    assert ok.all()
    assert np.array_equal(v_ref, v_orc), _ulps(v_ref, v_orc)


def test_shake_bit_exact_with_reference(pq, orc, ref, sysx):
    topo, _ = sysx
    x0 = topo.positions
    v = _thermal(topo, 4)
    dt = np.float32(0.004)
    x = (x0 + dt * v).astype(np.float32)  # the drift, as DRIFT_SAVE_XN computes it
    o = _orc(orc, topo)
    o.set_state(x, v)
    assert o.shake_all(x0) == 0  # converges on the CPU first
    x_orc, v_orc = o.get_state()
    o.close()
    x_ref, v_ref, ok = ref.shake(topo, x, x0, v, float(dt))
    assert ok.all()
    assert np.array_equal(x_ref, x_orc), _ulps(x_ref, x_orc)
    assert np.array_equal(v_ref, v_orc), _ulps(v_ref, v_orc)


def test_velocity_clamp_bit_exact_with_reference(pq, orc, ref, sysx):
    topo, x = sysx
    v = _thermal(topo, 6)
    v[::5] *= 40.0  # above 20 thermal speeds
    o = _orc(orc, topo)
    o.set_state(x, v)
    o.clamp_all()
    _, v_orc = o.get_state()
    o.close()
    v_ref = ref.clamp(v, topo.masses, 300.0)
    assert not np.array_equal(v_ref, v)
    assert np.array_equal(v_ref, v_orc)
