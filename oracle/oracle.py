"""ctypes wrapper of the CPU oracle (oracle/prismq_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline / reference leg.  The product
package never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
import threading

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "prismq_oracle.c"
HDR = HERE / "prismq_oracle.h"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

FLAGS = ["-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


GEN_SRC = [HERE / "gen_shim.cpp", HERE.parent / "prism-q_gb300" / "csrc" / "topology.cpp"]
GEN_LIB = BUILD / "liboracle_gen.so"
GEN_FLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> pathlib.Path:
    """Compile the oracle with gcc (no contraction, OpenMP), and its build of
    the input generator (build_gen)."""
    build_gen(force)
    deps = [SRC, HDR, HERE.parent / "include" / "prismq_md.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".so.{os.getpid()}.{threading.get_ident()}.tmp")
    cmd = ["gcc", *FLAGS, "-o", str(tmp), str(SRC), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_gen(force: bool = False) -> pathlib.Path:
    """The library's synthetic-system generator (host C++) compiled into the
    oracle's own shared object, so CPU legs build inputs without the product
    library."""
    deps = GEN_SRC + [HERE.parent / "prism-q_gb300" / "csrc" / "pq_host.h", HERE.parent / "include" / "prismq_md.h"]
    if not force and GEN_LIB.exists() and all(GEN_LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return GEN_LIB
    BUILD.mkdir(exist_ok=True)
    tmp = GEN_LIB.with_suffix(f".so.{os.getpid()}.{threading.get_ident()}.tmp")
    cmd = ["g++", *GEN_FLAGS, "-o", str(tmp), *map(str, GEN_SRC)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle generator build failed:\n{res.stderr}")
    os.replace(tmp, GEN_LIB)
    return GEN_LIB


_gen = None
_gen_lock = threading.Lock()


def _load_gen() -> ctypes.CDLL:
    G = ctypes.CDLL(str(build_gen()))
    G.orcgen_polyala.restype = ctypes.c_void_p
    G.orcgen_polyala.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    G.orcgen_view.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    G.orcgen_free.argtypes = [ctypes.c_void_p]
    return G


def polyala(n_chains: int, n_residues: int, seed: int, density: float = 0.0, box_edge: float = 0.0,
            compact: bool = True, stats: dict | None = None):
    """A synthetic system from the oracle's build of the generator: the same
    bits as the library's Topology.polyala / polyala_compact for the same
    arguments.  Returns the package's Topology (a numpy container)."""
    global _gen
    import importlib

    with _gen_lock:  # the first callers may come from several threads at once
        if _gen is None:
            _gen = _load_gen()
    G = _gen
    pkg = importlib.import_module("prism-q_gb300")
    st = (ctypes.c_double * 4)()
    err = ctypes.create_string_buffer(256)
    if not compact and not (density > 0.0):
        density = 0.03
    h = G.orcgen_polyala(n_chains, n_residues, seed, float(np.float32(density)), float(np.float32(box_edge)),
                            1 if compact else 0, st, err, 256)
    if not h:
        raise RuntimeError(err.value.decode())
    try:
        t = pkg.TopologyStruct()
        G.orcgen_view(h, ctypes.byref(t))
        topo = pkg.Topology.from_struct(t)
    finally:
        G.orcgen_free(h)
    if stats is not None:
        stats.update(iterations=int(st[0]), max_overlap=st[1], max_outside=st[2], min_nonbonded=st[3])
    return topo


class OrcParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_float), ("temperature", ctypes.c_float), ("gamma", ctypes.c_float),
                ("cutoff", ctypes.c_float), ("c1", ctypes.c_float), ("max_iter", ctypes.c_int),
                ("com_interval", ctypes.c_int), ("seed", ctypes.c_uint32), ("stream", ctypes.c_uint32)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(str(path))
        P = ctypes.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [P, ctypes.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [P]
        L.orc_n_atoms.argtypes = [P]
        L.orc_set_state.argtypes = [P, P, P]
        L.orc_get_state.argtypes = [P, P, P]
        L.orc_forces_ref_f32.argtypes = [P, P, P, ctypes.c_int]
        L.orc_forces_f64.argtypes = [P, P, P, ctypes.c_int]
        L.orc_forces_f64_rule.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int]
        L.orc_rattle_all.argtypes = [P]
        L.orc_shake_all.argtypes = [P, P]
        L.orc_kick_all.argtypes = [P, P]
        L.orc_clamp_all.argtypes = [P]
        L.orc_ou_all.argtypes = [P, P, ctypes.c_float]
        L.orc_ou_all.restype = None
        L.orc_term_forces.argtypes = [P, P, P, P]
        L.orc_phases.argtypes = [P, ctypes.c_int, P, ctypes.c_longlong]
        L.orc_com_remove.argtypes = [P]
        L.orc_protocol_eval.argtypes = [P, ctypes.c_longlong, P]
        L.orc_protocol_eval.restype = None
        L.orc_set_protocol.argtypes = [P, P, ctypes.c_longlong]
        L.orc_set_protocol.restype = None
        L.orc_run.argtypes = [P, ctypes.c_long, ctypes.c_int]
        L.orc_step_count.restype = ctypes.c_longlong
        L.orc_step_count.argtypes = [P]
        L.orc_pairs_ref27.restype = ctypes.c_long
        L.orc_pairs_ref27.argtypes = [ctypes.c_int, P, P, ctypes.c_float, P, P, P, ctypes.c_long,
                                      ctypes.POINTER(ctypes.c_int)]
        L.orc_pairs_brute.restype = ctypes.c_long
        L.orc_pairs_brute.argtypes = [ctypes.c_int, P, ctypes.c_float, P, P, P, ctypes.c_long]
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_normal3.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                  ctypes.c_uint32, P]
        L.orc_ref_exclusions.argtypes = [P, P, P, ctypes.c_long]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def philox(ctr, key) -> tuple[int, int, int, int]:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return tuple(int(v) for v in o)


def normal3(seed: int, stream: int, atom: int, step: int, purpose: int) -> np.ndarray:
    o = np.zeros(3, dtype=np.float32)
    lib().orc_normal3(seed, stream, atom, step, purpose, _ptr(o))
    return o


def _csr(excl_off, excl):
    if excl_off is None:
        return None, None
    return (np.ascontiguousarray(excl_off, dtype=np.int32), np.ascontiguousarray(excl, dtype=np.int32))


def pairs_ref27(pos: np.ndarray, grid_pos: np.ndarray | None = None, r2max: float = 144.0,
                excl_off=None, excl=None) -> tuple[np.ndarray, int]:
    """Reference cell-scheme pair set (i<j, sorted) and the maximum cell occupancy."""
    p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    g = p if grid_pos is None else np.ascontiguousarray(grid_pos, dtype=np.float32).reshape(-1, 3)
    eo, el = _csr(excl_off, excl)
    occ = ctypes.c_int(0)
    n = lib().orc_pairs_ref27(len(p), _ptr(p), _ptr(g), r2max, _ptr(eo), _ptr(el), None, 0, ctypes.byref(occ))
    out = np.zeros((max(n, 1), 2), dtype=np.int32)
    n2 = lib().orc_pairs_ref27(len(p), _ptr(p), _ptr(g), r2max, _ptr(eo), _ptr(el), _ptr(out), n,
                               ctypes.byref(occ))
    assert n2 == n
    return out[:n], occ.value


def pairs_brute(pos: np.ndarray, r2max: float = 144.0, excl_off=None, excl=None) -> np.ndarray:
    p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    eo, el = _csr(excl_off, excl)
    n = lib().orc_pairs_brute(len(p), _ptr(p), r2max, _ptr(eo), _ptr(el), None, 0)
    out = np.zeros((max(n, 1), 2), dtype=np.int32)
    lib().orc_pairs_brute(len(p), _ptr(p), r2max, _ptr(eo), _ptr(el), _ptr(out), n)
    return out[:n]


def protocol_eval(proto_struct, director_step: int):
    """(T, γ, dt, c1) of the oracle's director restatement; proto_struct is a
    prismq_protocol (ctypes)."""
    out = (ctypes.c_float * 4)()
    lib().orc_protocol_eval(ctypes.byref(proto_struct), int(director_step), out)
    return tuple(float(v) for v in out)


def c1_of(gamma: float, dt: float) -> float:
    """exp(-γ·dt/2) rounded to float, computed as the library computes it."""
    hd = np.float32(0.5) * np.float32(dt)
    arg = np.float32(-np.float32(gamma) * hd)
    return float(np.float32(np.exp(np.float64(arg))))


class OracleSystem:
    """Oracle copy of one system; `topo_struct` is a prismq_topology (ctypes) pointer."""

    def __init__(self, topo_struct, *, dt=0.004, temperature=300.0, gamma=1.0, cutoff=10.0,
                 max_iter=100, com_interval=100, seed=0x50524953, stream=0, c1=None):
        p = OrcParams(dt, temperature, gamma, cutoff, c1 if c1 is not None else c1_of(gamma, dt),
                      max_iter, com_interval, seed, stream)
        self._p = p
        self.h = lib().orc_create(ctypes.byref(topo_struct), ctypes.byref(p))
        self.n = lib().orc_n_atoms(self.h)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_protocol(self, proto_struct, origin: int) -> None:
        """Every step st then runs with the director's values at st - origin."""
        self._proto = proto_struct
        lib().orc_set_protocol(self.h, ctypes.byref(proto_struct) if proto_struct is not None else None,
                               int(origin))

    def set_state(self, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, dtype=np.float32).reshape(-1)
        va = None if v is None else np.ascontiguousarray(v, dtype=np.float32).reshape(-1)
        lib().orc_set_state(self.h, _ptr(xa), _ptr(va))

    def get_state(self):
        x = np.zeros((self.n, 3), dtype=np.float32)
        v = np.zeros((self.n, 3), dtype=np.float32)
        lib().orc_get_state(self.h, _ptr(x), _ptr(v))
        return x, v

    def forces_ref_f32(self, threads: int = 0):
        f = np.zeros((self.n, 3), dtype=np.float32)
        e = np.zeros(5, dtype=np.float64)
        rc = lib().orc_forces_ref_f32(self.h, _ptr(f), _ptr(e), threads)
        if rc:
            raise RuntimeError(f"oracle force error {rc}")
        return f, e

    def forces_f64(self, threads: int = 0, incl64: bool = False):
        """FP64 forces and energies; pairs enter by the FP32 r^2 rule, or by r^2
        in double with incl64 (the pair set of an FP64-everywhere run)."""
        f = np.zeros((self.n, 3), dtype=np.float64)
        e = np.zeros(5, dtype=np.float64)
        lib().orc_forces_f64_rule(self.h, _ptr(f), _ptr(e), threads, 1 if incl64 else 0)
        return f, e

    # single pieces on the current state (pins against the reference's own functions)
    def rattle_all(self) -> int:
        return lib().orc_rattle_all(self.h)

    def shake_all(self, x_start) -> int:
        xs = np.ascontiguousarray(x_start, dtype=np.float32).reshape(-1)
        return lib().orc_shake_all(self.h, _ptr(xs))

    def kick_all(self, f) -> None:
        fa = np.ascontiguousarray(f, dtype=np.float32).reshape(-1)
        lib().orc_kick_all(self.h, _ptr(fa))

    def clamp_all(self) -> None:
        lib().orc_clamp_all(self.h)

    def ou_all(self, z, c1: float) -> None:
        """One OU half-step of every atom with the given normals [n, 3] and c1."""
        za = np.ascontiguousarray(z, dtype=np.float32).reshape(-1)
        lib().orc_ou_all(self.h, _ptr(za), float(c1))

    def term_forces(self, nb: int, na: int, nd: int):
        fb = np.zeros((nb, 2, 3), np.float32)
        fa = np.zeros((na, 3, 3), np.float32)
        fd = np.zeros((nd, 4, 3), np.float32)
        lib().orc_term_forces(self.h, _ptr(fb), _ptr(fa), _ptr(fd))
        return fb, fa, fd

    def phases(self, which: int, f_fixed: np.ndarray, step: int) -> int:
        ff = np.ascontiguousarray(f_fixed, dtype=np.int64).reshape(-1)
        return lib().orc_phases(self.h, which, _ptr(ff), step)

    def com_remove(self):
        lib().orc_com_remove(self.h)

    def run(self, n_steps: int, threads: int = 0) -> int:
        return lib().orc_run(self.h, n_steps, threads)

    @property
    def step(self) -> int:
        return lib().orc_step_count(self.h)

    def ref_exclusions(self):
        off = np.zeros(self.n + 1, dtype=np.int32)
        cap = 64 * self.n + 1
        lst = np.zeros(cap, dtype=np.int32)
        tot = lib().orc_ref_exclusions(self.h, _ptr(off), _ptr(lst), cap)
        return off, lst[:tot]
