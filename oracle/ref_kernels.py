"""Host side of the reference-kernel harness — test infrastructure (oracle side).

Loads oracle/_ref/ref_harness*.cubin (built by oracle/build_ref.py from the
reference's own CUDA source) through the CUDA driver API (libcuda, ctypes) in
the device's primary context, and runs the wrappers of oracle/ref_harness.cu
on numpy arrays.  Every launch is one thread per term / cluster / atom with
a bounds check in the kernel; callers validate indices before calling.
"""
from __future__ import annotations

import ctypes
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
CUBIN = {False: HERE / "_ref" / "ref_harness.cubin", True: HERE / "_ref" / "ref_harness_nofma.cubin"}


def available() -> bool:
    return all(p.exists() for p in CUBIN.values())


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        c = self.cu
        c.cuInit.argtypes = [ctypes.c_uint]
        c.cuDeviceGet.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int]
        c.cuDevicePrimaryCtxRetain.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
        c.cuCtxSetCurrent.argtypes = [ctypes.c_void_p]
        c.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        c.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        c.cuMemAlloc_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
        c.cuMemFree_v2.argtypes = [ctypes.c_uint64]
        c.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]
        c.cuMemcpyDtoH_v2.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t]
        c.cuLaunchKernel.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        c.cuCtxSynchronize.argtypes = []
        self.check(c.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.check(c.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        ctx = ctypes.c_void_p()
        self.check(c.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self.check(c.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.mods: dict[bool, ctypes.c_void_p] = {}

    @staticmethod
    def check(rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUDA driver error {rc}")

    def module(self, nofma: bool) -> ctypes.c_void_p:
        if nofma not in self.mods:
            m = ctypes.c_void_p()
            self.check(self.cu.cuModuleLoad(ctypes.byref(m), str(CUBIN[nofma]).encode()), "cuModuleLoad")
            self.mods[nofma] = m
        return self.mods[nofma]

    def function(self, nofma: bool, name: str) -> ctypes.c_void_p:
        f = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.module(nofma), name.encode()), name)
        return f


_drv: _Driver | None = None


def _driver() -> _Driver:
    global _drv
    if _drv is None:
        _drv = _Driver()
    return _drv


class _Dev:
    """Device copies of numpy arrays for one launch."""

    def __init__(self):
        self.d = _driver()
        self.ptrs: list[int] = []

    def put(self, a: np.ndarray) -> ctypes.c_uint64:
        a = np.ascontiguousarray(a)
        p = ctypes.c_uint64()
        self.d.check(self.d.cu.cuMemAlloc_v2(ctypes.byref(p), max(a.nbytes, 16)), "cuMemAlloc")
        self.ptrs.append(p.value)
        if a.nbytes:
            self.d.check(self.d.cu.cuMemcpyHtoD_v2(p, a.ctypes.data, a.nbytes), "cuMemcpyHtoD")
        return p

    def get(self, p: ctypes.c_uint64, like: np.ndarray) -> np.ndarray:
        out = np.empty_like(like)
        if out.nbytes:
            self.d.check(self.d.cu.cuMemcpyDtoH_v2(out.ctypes.data, p, out.nbytes), "cuMemcpyDtoH")
        return out

    def launch(self, nofma: bool, name: str, n: int, args: list) -> None:
        f = self.d.function(nofma, name)
        holders = [a if isinstance(a, (ctypes.c_uint64, ctypes.c_int, ctypes.c_float)) else a for a in args]
        argv = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        blocks = max(1, (n + 127) // 128)
        self.d.check(self.d.cu.cuLaunchKernel(f, blocks, 1, 1, 128, 1, 1, 0, None, argv, None), name)
        self.d.check(self.d.cu.cuCtxSynchronize(), name + " (sync)")

    def free(self) -> None:
        for p in self.ptrs:
            self.d.cu.cuMemFree_v2(p)
        self.ptrs.clear()


def _i(v: int) -> ctypes.c_int:
    return ctypes.c_int(int(v))


def _f(v: float) -> ctypes.c_float:
    return ctypes.c_float(float(v))


def _pos3(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, 3))


def bond_terms(topo, x, nofma=False):
    """Per-term forces [nb, 2, 3] and energy shares [nb, 2] from compute_bond_force."""
    b = topo.bonds
    n = len(b)
    D = _Dev()
    try:
        ij = np.stack([b["i"], b["j"]], 1).astype(np.int32)
        p = np.stack([b["r0"], b["k"]], 1).astype(np.float32)
        out = np.zeros((n, 2, 3), np.float32)
        pe = np.zeros((n, 2), np.float64)
        d_out, d_pe = D.put(out), D.put(pe)
        D.launch(nofma, "refh_bonds", n, [_i(n), D.put(ij), D.put(p), D.put(_pos3(x)), d_out, d_pe])
        return D.get(d_out, out), D.get(d_pe, pe)
    finally:
        D.free()


def angle_terms(topo, x, nofma=False):
    a = topo.angles
    n = len(a)
    D = _Dev()
    try:
        ijk = np.stack([a["i"], a["j"], a["k"]], 1).astype(np.int32)
        p = np.stack([a["theta0"], a["force_k"]], 1).astype(np.float32)
        out = np.zeros((n, 3, 3), np.float32)
        pe = np.zeros((n, 3), np.float64)
        d_out, d_pe = D.put(out), D.put(pe)
        D.launch(nofma, "refh_angles", n, [_i(n), D.put(ijk), D.put(p), D.put(_pos3(x)), d_out, d_pe])
        return D.get(d_out, out), D.get(d_pe, pe)
    finally:
        D.free()


def dihedral_terms(topo, x, nofma=False):
    t = topo.dihedrals
    n = len(t)
    D = _Dev()
    try:
        ijkl = np.stack([t["i"], t["j"], t["k"], t["l"]], 1).astype(np.int32)
        per = np.ascontiguousarray(t["periodicity"].astype(np.int32))
        p = np.stack([t["phase"], t["force_k"]], 1).astype(np.float32)
        out = np.zeros((n, 4, 3), np.float32)
        pe = np.zeros((n, 4), np.float64)
        d_out, d_pe = D.put(out), D.put(pe)
        D.launch(nofma, "refh_dihedrals", n, [_i(n), D.put(ijkl), D.put(per), D.put(p), D.put(_pos3(x)), d_out,
                                              d_pe])
        return D.get(d_out, out), D.get(d_pe, pe)
    finally:
        D.free()


def pair_terms(topo, x, pairs, exact, ex_params, cutoff=10.0, nofma=False):
    """compute_nonbonded_force per pair: forces [n, 2, 3] and energy shares [n, 2]."""
    n = len(pairs)
    D = _Dev()
    try:
        out = np.zeros((n, 2, 3), np.float32)
        pe = np.zeros((n, 2), np.float64)
        d_out, d_pe = D.put(out), D.put(pe)
        D.launch(nofma, "refh_pairs", n,
                 [_i(n), D.put(np.asarray(pairs, np.int32)), D.put(np.asarray(exact, np.int32)),
                  D.put(np.asarray(ex_params, np.float32)), D.put(topo.charges.astype(np.float32)),
                  D.put(topo.lj_sigma.astype(np.float32)), D.put(topo.lj_epsilon.astype(np.float32)),
                  _f(np.float32(cutoff) * np.float32(cutoff)), D.put(_pos3(x)), d_out, d_pe])
        return D.get(d_out, out), D.get(d_pe, pe)
    finally:
        D.free()


def kick(v, f, mass, dt, exact, nofma=True):
    D = _Dev()
    try:
        vv = _pos3(v)
        d_v = D.put(vv)
        n = len(vv)
        D.launch(nofma, "refh_kick", n, [_i(n), d_v, D.put(_pos3(f)), D.put(np.asarray(mass, np.float32)), _f(dt),
                                        _i(1 if exact else 0)])
        return D.get(d_v, vv)
    finally:
        D.free()


def _clusters(topo):
    c = topo.clusters
    ci = np.stack([c["central_atom"], c["hydrogen_atoms"][:, 0], c["hydrogen_atoms"][:, 1],
                   c["hydrogen_atoms"][:, 2], c["n_hydrogens"]], 1).astype(np.int32)
    cf = np.stack([c["bond_lengths"][:, 0], c["bond_lengths"][:, 1], c["bond_lengths"][:, 2],
                   c["inv_mass_central"], c["inv_mass_h"]], 1).astype(np.float32)
    return ci, cf


def rattle(topo, x, v, max_iter=100, nofma=True):
    """rattle_cluster_velocities on every cluster; returns (v, ok[n_clusters])."""
    ci, cf = _clusters(topo)
    n = len(ci)
    D = _Dev()
    try:
        vv = _pos3(v)
        ok = np.zeros(n, np.int32)
        d_v, d_ok = D.put(vv), D.put(ok)
        D.launch(nofma, "refh_rattle", n, [_i(n), D.put(ci), D.put(cf), D.put(_pos3(x)), d_v, _i(max_iter), d_ok])
        return D.get(d_v, vv), D.get(d_ok, ok)
    finally:
        D.free()


def shake(topo, x, x0, v, dt, max_iter=100, step=0, nofma=True):
    """shake_cluster_positions on every cluster; returns (x, v, ok[n_clusters])."""
    ci, cf = _clusters(topo)
    n = len(ci)
    D = _Dev()
    try:
        xx, vv = _pos3(x), _pos3(v)
        ok = np.zeros(n, np.int32)
        d_x, d_v, d_ok = D.put(xx), D.put(vv), D.put(ok)
        D.launch(nofma, "refh_shake", n, [_i(n), D.put(ci), D.put(cf), d_x, D.put(_pos3(x0)), d_v, _f(dt),
                                         _i(max_iter), _i(step), d_ok])
        return D.get(d_x, xx), D.get(d_v, vv), D.get(d_ok, ok)
    finally:
        D.free()


def clamp(v, mass, temperature, nofma=True):
    """The reference's nhs_velocity_safety_clamp kernel as it is."""
    D = _Dev()
    try:
        size = np.zeros(1, np.int32)
        d_size = D.put(size)
        D.launch(nofma, "refh_protocol_size", 1, [d_size])
        nbytes = int(D.get(d_size, size)[0])
        d_proto = D.put(np.zeros(nbytes, np.uint8))
        D.launch(nofma, "refh_protocol_init", 1, [d_proto, _f(temperature)])
        vv = _pos3(v)
        n = len(vv)
        d_v = D.put(vv)
        D.launch(nofma, "nhs_velocity_safety_clamp", n,
                 [d_v, D.put(np.asarray(mass, np.float32)), _i(n), d_proto, ctypes.c_uint64(0)])
        return D.get(d_v, vv)
    finally:
        D.free()


def ou(v, mass, temperature, gamma, dt, seed, nofma=True):
    """One OU half-step by the reference's langevin_thermostat from cuRAND
    states initialised as init_rng_states does; returns (v, normals [n, 3],
    c1) with the normals the thermostat drew and its c1."""
    D = _Dev()
    try:
        vv = _pos3(v)
        n = len(vv)
        z = np.zeros((n, 3), np.float32)
        c1 = np.zeros(1, np.float32)
        d_v, d_z, d_c1 = D.put(vv), D.put(z), D.put(c1)
        D.launch(nofma, "refh_ou", n, [_i(n), d_v, D.put(np.asarray(mass, np.float32)), _f(temperature), _f(gamma),
                                      _f(dt), ctypes.c_uint64(int(seed)), d_z, d_c1])
        return D.get(d_v, vv), D.get(d_z, z), float(D.get(d_c1, c1)[0])
    finally:
        D.free()
