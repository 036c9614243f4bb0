"""GB300-native Prism-Q classical MD step — Python host API over the C ABI.

The compute path is libprismq_md.so (hand-written sm_103a CUDA, built in-tree
by build.py); this module is a thin ctypes layer that mirrors the reference
engine's interface (NhsAmberFusedEngine, crates/prism-nhs/src/fused_engine.rs:
new_on_stream :10800, set_dt :15342, step :18963, run :23911,
rebuild_neighbor_lists :16615, get_positions :24117, get_velocities :20939)
with the same argument meaning.  Errors raise PrismQError carrying the C
status code; there is no CPU fallback — without the built library or a GPU,
calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
from dataclasses import dataclass

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "libprismq_md.so"
HEADER = _HERE.parent / "include" / "prismq_md.h"

STATUS = {
    0: "OK", 1: "E_INVALID", 2: "E_CUDA", 3: "E_NO_DEVICE", 4: "E_CAPACITY", 5: "E_CELL_OVERFLOW",
    6: "E_NEIGHBOR_OVERFLOW", 7: "E_SHAKE", 8: "E_RATTLE", 9: "E_NONFINITE", 10: "E_BUSY",
    11: "E_NOT_FOUND",
}
NLIST_COMPLETE, NLIST_REF27 = 0, 1
PRECISION_FP32, PRECISION_FP64 = 0, 1
PHASES_PRE, PHASES_POST = 1, 2
PAIR_ROWS, PAIR_TILES = 0, 1


class PrismQError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


# ---------------------------------------------------------------- C structs
class Bond(ctypes.Structure):
    _fields_ = [("i", ctypes.c_int32), ("j", ctypes.c_int32), ("r0", ctypes.c_float), ("k", ctypes.c_float)]


class Angle(ctypes.Structure):
    _fields_ = [("i", ctypes.c_int32), ("j", ctypes.c_int32), ("k", ctypes.c_int32),
                ("theta0", ctypes.c_float), ("force_k", ctypes.c_float)]


class Dihedral(ctypes.Structure):
    _fields_ = [("i", ctypes.c_int32), ("j", ctypes.c_int32), ("k", ctypes.c_int32), ("l", ctypes.c_int32),
                ("periodicity", ctypes.c_int32), ("phase", ctypes.c_float), ("force_k", ctypes.c_float)]


class Exception14(ctypes.Structure):
    _fields_ = [("i", ctypes.c_int32), ("j", ctypes.c_int32), ("charge_product", ctypes.c_float),
                ("sigma", ctypes.c_float), ("epsilon", ctypes.c_float)]


class HCluster(ctypes.Structure):
    _fields_ = [("central_atom", ctypes.c_int32), ("hydrogen_atoms", ctypes.c_int32 * 3),
                ("bond_lengths", ctypes.c_float * 3), ("n_hydrogens", ctypes.c_int32),
                ("inv_mass_central", ctypes.c_float), ("inv_mass_h", ctypes.c_float)]


_P = ctypes.c_void_p


class TopologyStruct(ctypes.Structure):
    _fields_ = [("n_atoms", ctypes.c_int32), ("positions", _P), ("masses", _P), ("charges", _P),
                ("lj_sigma", _P), ("lj_epsilon", _P),
                ("n_bonds", ctypes.c_int32), ("bonds", _P), ("n_angles", ctypes.c_int32), ("angles", _P),
                ("n_dihedrals", ctypes.c_int32), ("dihedrals", _P),
                ("n_exceptions", ctypes.c_int32), ("exceptions", _P),
                ("exclusion_offsets", _P), ("exclusions", _P),
                ("n_clusters", ctypes.c_int32), ("clusters", _P)]


class ParamsStruct(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_float), ("temperature", ctypes.c_float), ("gamma", ctypes.c_float),
                ("cutoff", ctypes.c_float), ("skin", ctypes.c_float), ("rebuild_interval", ctypes.c_int32),
                ("com_interval", ctypes.c_int32), ("max_constraint_iter", ctypes.c_int32),
                ("seed", ctypes.c_uint32), ("stream", ctypes.c_uint32),
                ("shake_tol", ctypes.c_float), ("rattle_tol", ctypes.c_float),
                ("constraint_check_fp64", ctypes.c_int32), ("precision", ctypes.c_int32)]


class ProtocolStruct(ctypes.Structure):
    _fields_ = [("start_temp", ctypes.c_float), ("end_temp", ctypes.c_float),
                ("cold_hold_steps", ctypes.c_int32), ("ramp_steps", ctypes.c_int32),
                ("warm_hold_steps", ctypes.c_int32), ("ramp_down_steps", ctypes.c_int32),
                ("cold_return_steps", ctypes.c_int32), ("gamma_base", ctypes.c_float),
                ("cryo_enabled", ctypes.c_int32), ("equilibration_steps", ctypes.c_int32),
                ("equilibration_gamma", ctypes.c_float), ("adaptive_dt", ctypes.c_int32),
                ("base_dt", ctypes.c_float), ("current_step", ctypes.c_int32)]


class PrepOptionsStruct(ctypes.Structure):
    _fields_ = [("apply_hmr", ctypes.c_int32), ("require_harmonic_contract", ctypes.c_int32),
                ("require_exceptions", ctypes.c_int32), ("reserved", ctypes.c_int32), ("hmr_factor", ctypes.c_double)]


class PrepReportStruct(ctypes.Structure):
    _fields_ = [("hmr_performed", ctypes.c_int32), ("n_repartitioned", ctypes.c_int32),
                ("n_skipped", ctypes.c_int32), ("exact_exceptions", ctypes.c_int32),
                ("bond_scale", ctypes.c_double), ("angle_scale", ctypes.c_double),
                ("total_mass_before", ctypes.c_double), ("total_mass_after", ctypes.c_double)]


class ServerConfigStruct(ctypes.Structure):
    _fields_ = [("max_systems", ctypes.c_int32), ("chunk_steps", ctypes.c_int32), ("max_bypass_s", ctypes.c_double)]


class JobStruct(ctypes.Structure):
    _fields_ = [("topology", _P), ("params", ParamsStruct), ("n_steps", ctypes.c_int64),
                ("positions_out", _P), ("velocities_out", _P), ("tag", ctypes.c_uint64), ("protocol", _P),
                ("resume", _P), ("resume_len", ctypes.c_size_t), ("snapshot_out", _P),
                ("snapshot_cap", ctypes.c_size_t)]


class JobResultStruct(ctypes.Structure):
    _fields_ = [("job_id", ctypes.c_int64), ("tag", ctypes.c_uint64), ("status", ctypes.c_int),
                ("n_atoms", ctypes.c_int32), ("steps_done", ctypes.c_int64), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("end_s", ctypes.c_double), ("message", ctypes.c_char * 160),
                ("snapshot_len", ctypes.c_uint64)]


class ServerStatsStruct(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "queued", "resident_jobs",
                                                  "resident_atoms", "capacity_atoms", "device_bytes", "chunks")] + \
               [(n, ctypes.c_double) for n in ("atom_steps", "busy_s", "uptime_s")]


# numpy dtypes with the same layout as the C structs
BOND_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("r0", "<f4"), ("k", "<f4")])
ANGLE_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("theta0", "<f4"), ("force_k", "<f4")])
DIH_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("l", "<i4"), ("periodicity", "<i4"),
                   ("phase", "<f4"), ("force_k", "<f4")])
EXC_DT = np.dtype([("i", "<i4"), ("j", "<i4"), ("charge_product", "<f4"), ("sigma", "<f4"), ("epsilon", "<f4")])
CLUSTER_DT = np.dtype([("central_atom", "<i4"), ("hydrogen_atoms", "<i4", (3,)), ("bond_lengths", "<f4", (3,)),
                       ("n_hydrogens", "<i4"), ("inv_mass_central", "<f4"), ("inv_mass_h", "<f4")])

_lib = None


def load() -> ctypes.CDLL:
    """Load libprismq_md.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise PrismQError(2, f"{LIB_PATH} is not built; run prism-q_gb300/build.py")
    L = ctypes.CDLL(str(LIB_PATH))
    I, P, i64 = ctypes.c_int, ctypes.c_void_p, ctypes.c_int64
    sigs = {
        "prismq_last_error": (ctypes.c_char_p, []),
        "prismq_abi_version": (I, []),
        "prismq_device_count": (I, []),
        "prismq_kernel_launches": (ctypes.c_longlong, []),
        "prismq_set_device": (I, [ctypes.c_int32]),
        "prismq_batch_set_pair_layout": (I, [P, ctypes.c_int32]),
        "prismq_batch_pair_layout": (ctypes.c_int32, [P]),
        "prismq_set_pair_layout": (I, [P, ctypes.c_int32]),
        "prismq_device_ordinal": (ctypes.c_int32, []),
        "prismq_device_info": (I, [P]),
        "prismq_params_default": (None, [P]),
        "prismq_polyala_build": (I, [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float,
                                     ctypes.c_float, P]),
        "prismq_polyala_build_compact": (I, [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float,
                                             ctypes.c_float, P, P]),
        "prismq_topology_view": (I, [P, P]),
        "prismq_prep_options_default": (None, [P]),
        "prismq_protocol_default": (None, [P]),
        "prismq_protocol_eval": (I, [P, i64, P]),
        "prismq_set_protocol": (I, [P, P]),
        "prismq_get_step_params": (I, [P, P]),
        "prismq_batch_set_protocol": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_get_step_params": (I, [P, ctypes.c_int32, P]),
        "prismq_checkpoint_size": (I, [P, P]),
        "prismq_checkpoint_size_for_atoms": (I, [ctypes.c_int64, P]),
        "prismq_checkpoint_save": (I, [P, P, ctypes.c_size_t, P]),
        "prismq_checkpoint_restore": (I, [P, P, ctypes.c_size_t]),
        "prismq_batch_checkpoint_size": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_checkpoint_save": (I, [P, ctypes.c_int32, P, ctypes.c_size_t, P]),
        "prismq_batch_checkpoint_restore": (I, [P, ctypes.c_int32, P, ctypes.c_size_t]),
        "prismq_frames_configure": (I, [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
        "prismq_frames_read": (I, [P, P, P, P, ctypes.c_int32, P, P]),
        "prismq_batch_frames_configure": (I, [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
        "prismq_batch_frames_read": (I, [P, ctypes.c_int32, P, P, P, ctypes.c_int32, P, P]),
        "prismq_topology_from_prep_json": (I, [ctypes.c_char_p, ctypes.c_size_t, P, P, P]),
        "prismq_topology_load_prep_json": (I, [ctypes.c_char_p, P, P, P]),
        "prismq_topology_free": (None, [P]),
        "prismq_system_create": (I, [P, P, P]),
        "prismq_system_destroy": (None, [P]),
        "prismq_system_n_atoms": (ctypes.c_int32, [P]),
        "prismq_set_dt": (I, [P, ctypes.c_float]),
        "prismq_set_temperature": (I, [P, ctypes.c_float]),
        "prismq_set_gamma": (I, [P, ctypes.c_float]),
        "prismq_set_positions": (I, [P, P]),
        "prismq_set_velocities": (I, [P, P]),
        "prismq_get_positions": (I, [P, P]),
        "prismq_get_velocities": (I, [P, P]),
        "prismq_get_step": (I, [P, P]),
        "prismq_set_step": (I, [P, i64]),
        "prismq_compute_forces": (I, [P, P, P, P]),
        "prismq_energy_components": (I, [P, P]),
        "prismq_build_neighbors": (I, [P, I, P, ctypes.c_size_t, P]),
        "prismq_step": (I, [P, i64]),
        "prismq_debug_phases": (I, [P, I, i64]),
        "prismq_debug_noise": (None, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                      ctypes.c_uint32, P]),
        "prismq_batch_create": (I, [i64, ctypes.c_int32, P]),
        "prismq_batch_destroy": (None, [P]),
        "prismq_batch_add_system": (I, [P, P, P, P]),
        "prismq_batch_remove_system": (I, [P, ctypes.c_int32]),
        "prismq_batch_step": (I, [P, i64]),
        "prismq_batch_get_state": (I, [P, ctypes.c_int32, P, P]),
        "prismq_batch_set_state": (I, [P, ctypes.c_int32, P, P]),
        "prismq_batch_get_step": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_status": (I, [P, ctypes.c_int32]),
        "prismq_batch_energy": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_resident_atoms": (i64, [P]),
        "prismq_batch_resident_systems": (ctypes.c_int32, [P]),
        "prismq_batch_atom_span": (i64, [P]),
        "prismq_batch_atom_offset": (i64, [P, ctypes.c_int32]),
        "prismq_batch_set_state_all": (I, [P, P, P]),
        "prismq_batch_get_state_all": (I, [P, P, P]),
        "prismq_batch_step_host": (I, [P, ctypes.c_int64, P, P, P, P]),
        "prismq_batch_run_timed": (I, [P, i64, P, P]),
        "prismq_batch_time_force": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_counters": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_tuning": (I, [P, P]),
        "prismq_batch_set_force_variant": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_create_ex": (I, [i64, ctypes.c_int32, ctypes.c_int32, P]),
        "prismq_batch_virial": (I, [P, ctypes.c_int32, P]),
        "prismq_batch_get_state_f64": (I, [P, ctypes.c_int32, P, P]),
        "prismq_batch_get_forces_f64": (I, [P, ctypes.c_int32, P]),
        "prismq_virial": (I, [P, P]),
        "prismq_get_state_f64": (I, [P, P, P]),
        "prismq_get_forces_f64": (I, [P, P]),
        "prismq_server_config_default": (None, [P]),
        "prismq_server_create": (I, [i64, P, P]),
        "prismq_server_submit": (I, [P, P, P]),
        "prismq_server_poll": (I, [P, P, ctypes.c_int32, P, ctypes.c_int32]),
        "prismq_server_stats_get": (I, [P, P]),
        "prismq_server_destroy": (None, [P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != 0:
        msg = load().prismq_last_error()
        raise PrismQError(rc, msg.decode() if msg else "")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def device_count() -> int:
    return load().prismq_device_count()


def kernel_launches() -> int:
    return int(load().prismq_kernel_launches())


def set_device(ordinal: int) -> None:
    """Select the library's CUDA device for the calling thread (its runtime is
    its own: torch.cuda.set_device does not reach it)."""
    _check(load().prismq_set_device(int(ordinal)))


def device_ordinal() -> int:
    """The library's current device on the calling thread (-1 without one)."""
    return int(load().prismq_device_ordinal())


def device_info() -> dict:
    """{ordinal, sms, sm_clock_khz} of the library's current device."""
    out = (ctypes.c_int32 * 3)()
    _check(load().prismq_device_info(out))
    return {"ordinal": int(out[0]), "sms": int(out[1]), "sm_clock_khz": int(out[2])}


def debug_noise(seed: int, stream: int, atom: int, step: int, purpose: int) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    load().prismq_debug_noise(seed, stream, atom, step, purpose, _ptr(out))
    return out


# ---------------------------------------------------------------- parameters
@dataclass
class Params:
    dt: float = 0.004
    temperature: float = 300.0
    gamma: float = 1.0
    cutoff: float = 10.0
    skin: float = 2.0
    rebuild_interval: int = 20
    com_interval: int = 100
    max_constraint_iter: int = 100
    seed: int = 0x50524953
    stream: int = 0
    shake_tol: float = 1e-4           # |r^2 - L^2| / L^2 (reference value)
    rattle_tol: float = 1e-5          # relative velocity residual (reference value)
    constraint_check_fp64: bool = False
    precision: int = PRECISION_FP32   # PRECISION_FP64: FP64 state, forces and integrator

    def struct(self) -> ParamsStruct:
        return ParamsStruct(self.dt, self.temperature, self.gamma, self.cutoff, self.skin,
                            self.rebuild_interval, self.com_interval, self.max_constraint_iter,
                            self.seed & 0xffffffff, self.stream & 0xffffffff, self.shake_tol, self.rattle_tol,
                            1 if self.constraint_check_fp64 else 0, int(self.precision))


@dataclass
class Protocol:
    """Per-step temperature / friction / timestep schedule (ProtocolState,
    protocol_state.cuh:14-62; director protocol_director.cu:54-143).  The
    defaults are the physiological protocol with the reference's 10000-step
    friction blend from 1000 ps^-1."""
    start_temp: float = 300.0
    end_temp: float = 300.0
    cold_hold_steps: int = 0
    ramp_steps: int = 0
    warm_hold_steps: int = 100000
    ramp_down_steps: int = 0
    cold_return_steps: int = 0
    gamma_base: float = 1.0
    cryo_enabled: bool = False
    equilibration_steps: int = 10000
    equilibration_gamma: float = 1000.0
    adaptive_dt: int = 0            # 1: ramps at base_dt/2; 2: holds at 1.5 base_dt
    base_dt: float = 0.004
    current_step: int = 0

    def struct(self) -> ProtocolStruct:
        return ProtocolStruct(self.start_temp, self.end_temp, self.cold_hold_steps, self.ramp_steps,
                              self.warm_hold_steps, self.ramp_down_steps, self.cold_return_steps, self.gamma_base,
                              1 if self.cryo_enabled else 0, self.equilibration_steps, self.equilibration_gamma,
                              int(self.adaptive_dt), self.base_dt, self.current_step)

    def eval(self, director_step: int) -> tuple[float, float, float]:
        """(T, γ, dt) at one director step, computed by the library."""
        out = (ctypes.c_float * 3)()
        ps = self.struct()
        _check(load().prismq_protocol_eval(ctypes.byref(ps), int(director_step), out))
        return float(out[0]), float(out[1]), float(out[2])


# ---------------------------------------------------------------- topology
class Topology:
    """Owned numpy copy of a prismq_topology (PrismPrepTopology field set)."""

    def __init__(self, positions, masses, charges, lj_sigma, lj_epsilon, bonds=None, angles=None,
                 dihedrals=None, exceptions=None, exclusion_offsets=None, exclusions=None, clusters=None):
        self.positions = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        n = len(self.positions)
        self.masses = np.ascontiguousarray(masses, dtype=np.float32).reshape(n)
        self.charges = np.ascontiguousarray(charges, dtype=np.float32).reshape(n)
        self.lj_sigma = np.ascontiguousarray(lj_sigma, dtype=np.float32).reshape(n)
        self.lj_epsilon = np.ascontiguousarray(lj_epsilon, dtype=np.float32).reshape(n)
        self.bonds = np.ascontiguousarray(bonds if bonds is not None else np.zeros(0, BOND_DT), dtype=BOND_DT)
        self.angles = np.ascontiguousarray(angles if angles is not None else np.zeros(0, ANGLE_DT), dtype=ANGLE_DT)
        self.dihedrals = np.ascontiguousarray(dihedrals if dihedrals is not None else np.zeros(0, DIH_DT),
                                              dtype=DIH_DT)
        self.exceptions = np.ascontiguousarray(exceptions if exceptions is not None else np.zeros(0, EXC_DT),
                                               dtype=EXC_DT)
        if exclusion_offsets is None:
            exclusion_offsets = np.zeros(n + 1, np.int32)
            exclusions = np.zeros(0, np.int32)
        self.exclusion_offsets = np.ascontiguousarray(exclusion_offsets, dtype=np.int32)
        self.exclusions = np.ascontiguousarray(exclusions, dtype=np.int32)
        self.clusters = np.ascontiguousarray(clusters if clusters is not None else np.zeros(0, CLUSTER_DT),
                                             dtype=CLUSTER_DT)

    @property
    def n_atoms(self) -> int:
        return len(self.positions)

    def struct(self) -> TopologyStruct:
        t = TopologyStruct()
        t.n_atoms = self.n_atoms
        t.positions, t.masses, t.charges = _ptr(self.positions), _ptr(self.masses), _ptr(self.charges)
        t.lj_sigma, t.lj_epsilon = _ptr(self.lj_sigma), _ptr(self.lj_epsilon)
        t.n_bonds, t.bonds = len(self.bonds), _ptr(self.bonds)
        t.n_angles, t.angles = len(self.angles), _ptr(self.angles)
        t.n_dihedrals, t.dihedrals = len(self.dihedrals), _ptr(self.dihedrals)
        t.n_exceptions, t.exceptions = len(self.exceptions), _ptr(self.exceptions)
        t.exclusion_offsets, t.exclusions = _ptr(self.exclusion_offsets), _ptr(self.exclusions)
        t.n_clusters, t.clusters = len(self.clusters), _ptr(self.clusters)
        return t

    @classmethod
    def _from_buf(cls, buf) -> "Topology":
        """Copy the arrays of a prismq_topology_buf (the caller frees it)."""
        L = load()
        t = TopologyStruct()
        _check(L.prismq_topology_view(buf, ctypes.byref(t)))
        return cls.from_struct(t)

    @classmethod
    def from_struct(cls, t: TopologyStruct) -> "Topology":
        """Copy the arrays a prismq_topology points at."""
        n = t.n_atoms

        def arr(ptr, count, dtype, shape=None):
            if count == 0:
                return np.zeros(shape or 0, dtype=dtype)
            nbytes = count * np.dtype(dtype).itemsize
            raw = ctypes.string_at(ptr, nbytes)
            a = np.frombuffer(raw, dtype=dtype).copy()
            return a.reshape(shape) if shape else a

        eoff = arr(t.exclusion_offsets, n + 1, np.int32)
        return cls(arr(t.positions, 3 * n, np.float32, (n, 3)), arr(t.masses, n, np.float32),
                   arr(t.charges, n, np.float32), arr(t.lj_sigma, n, np.float32),
                   arr(t.lj_epsilon, n, np.float32), arr(t.bonds, t.n_bonds, BOND_DT),
                   arr(t.angles, t.n_angles, ANGLE_DT), arr(t.dihedrals, t.n_dihedrals, DIH_DT),
                   arr(t.exceptions, t.n_exceptions, EXC_DT), eoff,
                   arr(t.exclusions, int(eoff[-1]), np.int32), arr(t.clusters, t.n_clusters, CLUSTER_DT))

    @classmethod
    def polyala(cls, n_chains: int = 1, n_residues: int = 250, seed: int = 1, density: float = 0.03,
                box_edge: float = 0.0) -> "Topology":
        """Seeded synthetic poly-alanine-like system (C generator in the library)."""
        L = load()
        buf = ctypes.c_void_p()
        _check(L.prismq_polyala_build(n_chains, n_residues, seed, density, box_edge, ctypes.byref(buf)))
        try:
            return cls._from_buf(buf)
        finally:
            L.prismq_topology_free(buf)

    @classmethod
    def polyala_compact(cls, n_chains: int = 1, n_residues: int = 250, seed: int = 1, density: float = 0.0,
                        box_edge: float = 0.0, stats: dict | None = None) -> "Topology":
        """Seeded chains collapsed into a globule (one sphere per chain at `density`
        atoms/Å^3, 0 selects 0.0746: 2,500 atoms in a 40 Å globule) or packed into a
        cube of edge `box_edge` (prismq_polyala_build_compact).  `stats`, when given,
        receives the relaxation's iterations, overlap, wall violation and closest
        non-bonded distance."""
        L = load()
        buf = ctypes.c_void_p()
        st = (ctypes.c_double * 4)()
        _check(L.prismq_polyala_build_compact(n_chains, n_residues, seed, density, box_edge, st, ctypes.byref(buf)))
        if stats is not None:
            stats.update(iterations=int(st[0]), max_overlap=st[1], max_outside=st[2], min_nonbonded=st[3])
        try:
            return cls._from_buf(buf)
        finally:
            L.prismq_topology_free(buf)

    @classmethod
    def from_prep_json(cls, source, apply_hmr: bool = True, hmr_factor: float = 3.0,
                       require_harmonic_contract: bool = True, require_exceptions: bool = True,
                       report: dict | None = None) -> "Topology":
        """A PRISM-PREP topology JSON (PrismPrepTopology, input.rs:1027-1140) lowered for the engine.

        `source` is a path or the JSON text (str / bytes).  Validation, harmonic
        lowering and hydrogen mass repartitioning run in the library; a
        violated rule raises PrismQError with the rule named.  When `report`
        is a dict it receives what the load did (HMR, scales, mass totals)."""
        L = load()
        opt = PrepOptionsStruct()
        L.prismq_prep_options_default(ctypes.byref(opt))
        opt.apply_hmr, opt.hmr_factor = int(bool(apply_hmr)), float(hmr_factor)
        opt.require_harmonic_contract = int(bool(require_harmonic_contract))
        opt.require_exceptions = int(bool(require_exceptions))
        rep = PrepReportStruct()
        buf = ctypes.c_void_p()
        is_text = isinstance(source, (bytes, bytearray)) or (isinstance(source, str) and source.lstrip().startswith("{"))
        if is_text:
            data = source.encode() if isinstance(source, str) else bytes(source)
            _check(L.prismq_topology_from_prep_json(data, len(data), ctypes.byref(opt), ctypes.byref(buf),
                                                    ctypes.byref(rep)))
        else:
            _check(L.prismq_topology_load_prep_json(os.fsencode(source), ctypes.byref(opt), ctypes.byref(buf),
                                                    ctypes.byref(rep)))
        try:
            topo = cls._from_buf(buf)
        finally:
            L.prismq_topology_free(buf)
        if report is not None:
            report.update({f: getattr(rep, f) for f, _ in PrepReportStruct._fields_})
        return topo

    @classmethod
    def point_cloud(cls, positions) -> "Topology":
        """Atoms only (no bonded terms, exclusions or constraints): for neighbour-list parity."""
        p = np.asarray(positions, dtype=np.float32).reshape(-1, 3)
        n = len(p)
        return cls(p, np.full(n, 12.0, np.float32), np.zeros(n, np.float32), np.full(n, 3.0, np.float32),
                   np.full(n, 0.1, np.float32))


def _read_frames(call, n_atoms: int, velocities: bool, max_frames: int, chunk: int = 64) -> dict:
    xs, vs, steps, dropped = [], [], [], 0
    while len(steps) < max_frames:
        want = min(chunk, max_frames - len(steps))
        x = np.zeros((want, n_atoms, 3), np.float32)
        v = np.zeros((want, n_atoms, 3), np.float32) if velocities else None
        st = np.zeros(want, np.int64)
        got, lost = ctypes.c_int32(), ctypes.c_int64()
        _check(call(_ptr(x), _ptr(v) if v is not None else None, _ptr(st), want, ctypes.byref(got),
                    ctypes.byref(lost)))
        dropped += lost.value
        k = got.value
        xs.append(x[:k])
        if v is not None:
            vs.append(v[:k])
        steps.extend(st[:k].tolist())
        if k < want:
            break
    return {"steps": np.array(steps, np.int64), "positions": np.concatenate(xs) if xs else np.zeros((0, n_atoms, 3)),
            "velocities": (np.concatenate(vs) if vs else None), "dropped": dropped}


# ---------------------------------------------------------------- engine
class NhsAmberFusedEngine:
    """One system on the GPU (the drop-in for the reference engine's MD step)."""

    def __init__(self, topology: Topology, params: Params | None = None):
        self.topology = topology
        self.params = params or Params()
        self._t = topology.struct()
        self._p = self.params.struct()
        self.h = ctypes.c_void_p()
        _check(load().prismq_system_create(ctypes.byref(self._t), ctypes.byref(self._p), ctypes.byref(self.h)))
        self.n_atoms = topology.n_atoms

    # reference name: new_on_stream
    @classmethod
    def new_on_stream(cls, topology: Topology, params: Params | None = None) -> "NhsAmberFusedEngine":
        return cls(topology, params)

    def close(self) -> None:
        if self.h:
            load().prismq_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_dt(self, dt: float) -> None:
        _check(load().prismq_set_dt(self.h, dt))

    def set_temperature(self, t: float) -> None:
        _check(load().prismq_set_temperature(self.h, t))

    def set_gamma(self, g: float) -> None:
        _check(load().prismq_set_gamma(self.h, g))

    def set_protocol(self, protocol: "Protocol | None") -> None:
        """Install a run protocol (set_cryo_uv_protocol, fused_engine.rs:18815); None removes it."""
        ps = protocol.struct() if protocol is not None else None
        _check(load().prismq_set_protocol(self.h, ctypes.byref(ps) if ps is not None else None))

    def step_params(self) -> tuple[float, float, float]:
        """(T, γ, dt) of the next step."""
        out = (ctypes.c_float * 3)()
        _check(load().prismq_get_step_params(self.h, out))
        return float(out[0]), float(out[1]), float(out[2])

    def checkpoint(self) -> bytes:
        """The system's dynamic state at this step boundary (restore() resumes it bit for bit)."""
        L = load()
        n = ctypes.c_size_t()
        _check(L.prismq_checkpoint_size(self.h, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(L.prismq_checkpoint_save(self.h, buf, n.value, None))
        return buf.raw

    def restore(self, blob: bytes) -> None:
        _check(load().prismq_checkpoint_restore(self.h, blob, len(blob)))

    def record_frames(self, interval: int, capacity: int = 64, velocities: bool = False) -> None:
        """Record the state every `interval` steps into a device ring of `capacity` frames (0 stops)."""
        _check(load().prismq_frames_configure(self.h, interval, capacity, 1 if velocities else 0))
        self._frame_vel = velocities

    def read_frames(self, max_frames: int = 1 << 30):
        """Frames not yet read, oldest first: dict(steps, positions [F,N,3], velocities or None, dropped)."""
        return _read_frames(lambda *a: load().prismq_frames_read(self.h, *a), self.n_atoms,
                            getattr(self, "_frame_vel", False), max_frames)

    def save_checkpoint(self, path) -> None:
        pathlib.Path(path).write_bytes(self.checkpoint())

    def load_checkpoint(self, path) -> None:
        self.restore(pathlib.Path(path).read_bytes())

    def step(self, n_steps: int = 1) -> None:
        _check(load().prismq_step(self.h, n_steps))

    def run(self, n_steps: int) -> None:
        self.step(n_steps)

    @property
    def timestep(self) -> int:
        v = ctypes.c_int64()
        _check(load().prismq_get_step(self.h, ctypes.byref(v)))
        return v.value

    def set_timestep(self, step: int) -> None:
        _check(load().prismq_set_step(self.h, step))

    def get_positions(self) -> np.ndarray:
        out = np.zeros((self.n_atoms, 3), np.float32)
        _check(load().prismq_get_positions(self.h, _ptr(out)))
        return out

    def get_velocities(self) -> np.ndarray:
        out = np.zeros((self.n_atoms, 3), np.float32)
        _check(load().prismq_get_velocities(self.h, _ptr(out)))
        return out

    def set_positions(self, xyz) -> None:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1)
        _check(load().prismq_set_positions(self.h, _ptr(a)))

    def set_velocities(self, vxyz) -> None:
        a = np.ascontiguousarray(vxyz, dtype=np.float32).reshape(-1)
        _check(load().prismq_set_velocities(self.h, _ptr(a)))

    def compute_forces(self):
        """(pe_total, forces float[N,3], forces_fixed int64[N,3]) at the current positions."""
        pe = ctypes.c_double()
        f = np.zeros((self.n_atoms, 3), np.float32)
        fx = np.zeros((self.n_atoms, 3), np.int64)
        _check(load().prismq_compute_forces(self.h, ctypes.byref(pe), _ptr(f), _ptr(fx)))
        return pe.value, f, fx

    def energy_components(self) -> np.ndarray:
        """[bond, angle, dihedral, exception, nonbonded, kinetic] in kcal/mol (FP64)."""
        out = np.zeros(6, np.float64)
        _check(load().prismq_energy_components(self.h, _ptr(out)))
        return out

    def virial(self) -> np.ndarray:
        """W_ab = sum_i x_a F_b (3x3, kcal/mol), reduced in FP64."""
        out = np.zeros(9, np.float64)
        _check(load().prismq_virial(self.h, _ptr(out)))
        return out.reshape(3, 3)

    def get_state_f64(self):
        """(positions, velocities) as float64 [N,3] (native for FP64 systems)."""
        x = np.zeros((self.n_atoms, 3), np.float64)
        v = np.zeros((self.n_atoms, 3), np.float64)
        _check(load().prismq_get_state_f64(self.h, _ptr(x), _ptr(v)))
        return x, v

    def get_forces_f64(self) -> np.ndarray:
        """Forces of the last evaluation as float64 [N,3]."""
        f = np.zeros((self.n_atoms, 3), np.float64)
        _check(load().prismq_get_forces_f64(self.h, _ptr(f)))
        return f

    def build_neighbors(self, mode: int = NLIST_COMPLETE) -> np.ndarray:
        n = ctypes.c_size_t()
        L = load()
        rc = L.prismq_build_neighbors(self.h, mode, None, 0, ctypes.byref(n))
        if rc not in (0, 4):
            _check(rc)
        out = np.zeros((max(n.value, 1), 2), np.int32)
        _check(L.prismq_build_neighbors(self.h, mode, _ptr(out), n.value, ctypes.byref(n)))
        return out[: n.value]

    def rebuild_neighbor_lists(self) -> np.ndarray:
        return self.build_neighbors(NLIST_REF27)

    def set_pair_layout(self, layout: int) -> None:
        """PAIR_ROWS (default) or PAIR_TILES for the production list; set before stepping."""
        _check(load().prismq_set_pair_layout(self.h, int(layout)))

    def debug_phases(self, which: int, step: int) -> None:
        _check(load().prismq_debug_phases(self.h, which, step))


class Batch:
    """Many independent systems advanced together in one launch per phase."""

    def __init__(self, max_atoms: int, max_systems: int, precision: int = PRECISION_FP32):
        self.h = ctypes.c_void_p()
        _check(load().prismq_batch_create_ex(max_atoms, max_systems, precision, ctypes.byref(self.h)))
        self.n_atoms: dict[int, int] = {}
        self._keep: dict[int, tuple] = {}

    def close(self) -> None:
        if self.h:
            load().prismq_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_system(self, topology: Topology, params: Params | None = None) -> int:
        t = topology.struct()
        p = (params or Params()).struct()
        slot = ctypes.c_int32()
        _check(load().prismq_batch_add_system(self.h, ctypes.byref(t), ctypes.byref(p), ctypes.byref(slot)))
        self.n_atoms[slot.value] = topology.n_atoms
        return slot.value

    def remove_system(self, slot: int) -> None:
        _check(load().prismq_batch_remove_system(self.h, slot))
        self.n_atoms.pop(slot, None)

    def step(self, n_steps: int = 1) -> None:
        _check(load().prismq_batch_step(self.h, n_steps))

    def get_state(self, slot: int):
        n = self.n_atoms[slot]
        x = np.zeros((n, 3), np.float32)
        v = np.zeros((n, 3), np.float32)
        _check(load().prismq_batch_get_state(self.h, slot, _ptr(x), _ptr(v)))
        return x, v

    def set_state(self, slot: int, x=None, v=None) -> None:
        xa = None if x is None else np.ascontiguousarray(x, np.float32).reshape(-1)
        va = None if v is None else np.ascontiguousarray(v, np.float32).reshape(-1)
        _check(load().prismq_batch_set_state(self.h, slot, _ptr(xa), _ptr(va)))

    def timestep(self, slot: int) -> int:
        v = ctypes.c_int64()
        _check(load().prismq_batch_get_step(self.h, slot, ctypes.byref(v)))
        return v.value

    def status(self, slot: int) -> int:
        return load().prismq_batch_status(self.h, slot)

    def set_protocol(self, slot: int, protocol: "Protocol | None") -> None:
        ps = protocol.struct() if protocol is not None else None
        _check(load().prismq_batch_set_protocol(self.h, slot, ctypes.byref(ps) if ps is not None else None))

    def step_params(self, slot: int) -> tuple[float, float, float]:
        out = (ctypes.c_float * 3)()
        _check(load().prismq_batch_get_step_params(self.h, slot, out))
        return float(out[0]), float(out[1]), float(out[2])

    def checkpoint(self, slot: int) -> bytes:
        L = load()
        n = ctypes.c_size_t()
        _check(L.prismq_batch_checkpoint_size(self.h, slot, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(L.prismq_batch_checkpoint_save(self.h, slot, buf, n.value, None))
        return buf.raw

    def restore(self, slot: int, blob: bytes) -> None:
        _check(load().prismq_batch_checkpoint_restore(self.h, slot, blob, len(blob)))

    def record_frames(self, slot: int, interval: int, capacity: int = 64, velocities: bool = False) -> None:
        _check(load().prismq_batch_frames_configure(self.h, slot, interval, capacity, 1 if velocities else 0))
        self._frame_cfg = getattr(self, "_frame_cfg", {})
        self._frame_cfg[slot] = velocities

    def read_frames(self, slot: int, n_atoms: int, max_frames: int = 1 << 30):
        vel = getattr(self, "_frame_cfg", {}).get(slot, False)
        return _read_frames(lambda *a: load().prismq_batch_frames_read(self.h, slot, *a), n_atoms, vel, max_frames)

    def tuning(self) -> dict:
        """The autotuner's force-kernel launch shape for this batch."""
        out = np.zeros(5, np.int32)
        _check(load().prismq_batch_tuning_ex(self.h, _ptr(out)))
        return {"variant": int(out[0]), "block": int(out[1]), "atoms_per_block": int(out[3]),
                "min_blocks_per_sm": int(out[2]), "row_prefetch": int(out[4])}

    def atom_span(self) -> int:
        """Length (atoms) of the whole-arena state arrays."""
        return int(load().prismq_batch_atom_span(self.h))

    def atom_offset(self, slot: int) -> int:
        """First arena atom of a resident system."""
        return int(load().prismq_batch_atom_offset(self.h, slot))

    def get_state_all(self, xyz: np.ndarray | None = None, vxyz: np.ndarray | None = None):
        """Fill float32 [3 * atom_span] arrays (pinned host memory is written
        directly by the device; allocates pageable arrays when none are given)."""
        n = 3 * self.atom_span()
        if xyz is None and vxyz is None:
            xyz, vxyz = np.empty(n, np.float32), np.empty(n, np.float32)
        for a in (xyz, vxyz):
            if a is not None and (a.dtype != np.float32 or a.size != n or not a.flags.c_contiguous):
                raise ValueError(f"state arrays must be contiguous float32 of {n} values")
        _check(load().prismq_batch_get_state_all(self.h, _ptr(xyz), _ptr(vxyz)))
        return xyz, vxyz

    def set_state_all(self, xyz: np.ndarray | None, vxyz: np.ndarray | None) -> None:
        """Upload whole-arena state (float32 [3 * atom_span]; None leaves it)."""
        n = 3 * self.atom_span()
        for a in (xyz, vxyz):
            if a is not None and (a.dtype != np.float32 or a.size != n or not a.flags.c_contiguous):
                raise ValueError(f"state arrays must be contiguous float32 of {n} values")
        _check(load().prismq_batch_set_state_all(self.h, _ptr(xyz), _ptr(vxyz)))

    def step_host(self, n_steps: int, xyz_in, vxyz_in, xyz_out, vxyz_out) -> None:
        """Upload whole-arena state, step, and read it back in one call (one
        wait); arrays are float32 [3 * atom_span] or None."""
        n = 3 * self.atom_span()
        for a in (xyz_in, vxyz_in, xyz_out, vxyz_out):
            if a is not None and (a.dtype != np.float32 or a.size != n or not a.flags.c_contiguous):
                raise ValueError(f"state arrays must be contiguous float32 of {n} values")
        _check(load().prismq_batch_step_host(self.h, int(n_steps), _ptr(xyz_in), _ptr(vxyz_in), _ptr(xyz_out),
                                             _ptr(vxyz_out)))

    def set_pair_layout(self, layout: int) -> None:
        """PAIR_ROWS (default) or PAIR_TILES for the production list; set before stepping."""
        _check(load().prismq_batch_set_pair_layout(self.h, int(layout)))

    @property
    def pair_layout(self) -> int:
        return int(load().prismq_batch_pair_layout(self.h))

    def set_force_variant(self, variant: int) -> int:
        """Pin the force kernel's launch shape (-1: autotune); returns the number of shapes."""
        n = ctypes.c_int32()
        _check(load().prismq_batch_set_force_variant(self.h, int(variant), ctypes.byref(n)))
        return n.value

    def counters(self, slot: int) -> tuple[int, int]:
        """(steps taken, neighbour-list builds) of one system."""
        out = np.zeros(2, np.int64)
        _check(load().prismq_batch_counters(self.h, slot, _ptr(out)))
        return int(out[0]), int(out[1])

    def energy(self, slot: int) -> np.ndarray:
        out = np.zeros(6, np.float64)
        _check(load().prismq_batch_energy(self.h, slot, _ptr(out)))
        return out

    def virial(self, slot: int) -> np.ndarray:
        """W_ab = sum_i x_a F_b (3x3, kcal/mol) at the current positions."""
        out = np.zeros(9, np.float64)
        _check(load().prismq_batch_virial(self.h, slot, _ptr(out)))
        return out.reshape(3, 3)

    def get_state_f64(self, slot: int):
        n = self.n_atoms[slot]
        x = np.zeros((n, 3), np.float64)
        v = np.zeros((n, 3), np.float64)
        _check(load().prismq_batch_get_state_f64(self.h, slot, _ptr(x), _ptr(v)))
        return x, v

    def forces_f64(self, slot: int) -> np.ndarray:
        """Forces of the last evaluation (kcal/mol/Å) as float64."""
        f = np.zeros((self.n_atoms[slot], 3), np.float64)
        _check(load().prismq_batch_get_forces_f64(self.h, slot, _ptr(f)))
        return f

    @property
    def resident_atoms(self) -> int:
        return int(load().prismq_batch_resident_atoms(self.h))

    @property
    def resident_systems(self) -> int:
        return int(load().prismq_batch_resident_systems(self.h))


# ---------------------------------------------------------------- job server
@dataclass
class JobResult:
    job_id: int
    tag: int
    status: int
    n_atoms: int
    steps_done: int
    submit_s: float
    start_s: float
    end_s: float
    message: str
    positions: np.ndarray | None
    velocities: np.ndarray | None
    snapshot: bytes | None = None

    @property
    def latency_s(self) -> float:
        return self.end_s - self.submit_s

    @property
    def ok(self) -> bool:
        return self.status == 0


class Server:
    """Continuous-batching MD job server (prismq_server_*): one worker thread
    owns a device arena of at most max_hbm_bytes, admits queued jobs as arena
    space frees up and advances every resident job together."""

    def __init__(self, max_hbm_bytes: int, max_systems: int = 1024, chunk_steps: int = 50,
                 max_bypass_s: float = 1.0):
        cfg = ServerConfigStruct(max_systems, chunk_steps, max_bypass_s)
        self.h = ctypes.c_void_p()
        _check(load().prismq_server_create(int(max_hbm_bytes), ctypes.byref(cfg), ctypes.byref(self.h)))
        self._out: dict[int, tuple] = {}

    def close(self) -> None:
        if self.h:
            load().prismq_server_destroy(self.h)
            self.h = None
            self._out.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, topology: Topology, n_steps: int, params: Params | None = None, tag: int = 0,
               want_state: bool = True, protocol: "Protocol | None" = None, resume: bytes | None = None,
               want_snapshot: bool = False) -> int:
        """Queue a job.  ``resume`` is a checkpoint of this topology to start
        from (a job's snapshot or an engine's checkpoint); ``want_snapshot``
        returns the job's final checkpoint in ``JobResult.snapshot``."""
        n = topology.n_atoms
        x = np.zeros((n, 3), np.float32) if want_state else None
        v = np.zeros((n, 3), np.float32) if want_state else None
        t = topology.struct()
        ps = protocol.struct() if protocol is not None else None
        snap = None
        if want_snapshot:
            size = ctypes.c_size_t()
            _check(load().prismq_checkpoint_size_for_atoms(int(n), ctypes.byref(size)))
            snap = ctypes.create_string_buffer(size.value)
        rb = bytes(resume) if resume is not None else None
        job = JobStruct(ctypes.cast(ctypes.pointer(t), _P), (params or Params()).struct(), int(n_steps),
                        _ptr(x), _ptr(v), int(tag) & 0xffffffffffffffff,
                        ctypes.cast(ctypes.pointer(ps), _P) if ps is not None else None,
                        ctypes.cast(ctypes.c_char_p(rb), _P) if rb else None, len(rb) if rb else 0,
                        ctypes.cast(snap, _P) if snap is not None else None,
                        ctypes.sizeof(snap) if snap is not None else 0)
        jid = ctypes.c_int64()
        _check(load().prismq_server_submit(self.h, ctypes.byref(job), ctypes.byref(jid)))
        self._out[jid.value] = (x, v, snap)  # the worker writes here when the job ends
        return jid.value

    def poll(self, wait_ms: int = 0, max_results: int = 256) -> list[JobResult]:
        buf = (JobResultStruct * max_results)()
        n = ctypes.c_int32()
        _check(load().prismq_server_poll(self.h, buf, max_results, ctypes.byref(n), int(wait_ms)))
        out = []
        for r in buf[:n.value]:
            x, v, snap = self._out.pop(r.job_id, (None, None, None))
            blob = snap.raw[:r.snapshot_len] if snap is not None and r.snapshot_len else None
            out.append(JobResult(r.job_id, r.tag, r.status, r.n_atoms, r.steps_done, r.submit_s, r.start_s,
                                 r.end_s, r.message.decode(errors="replace"), x, v, blob))
        return out

    def stats(self) -> dict:
        st = ServerStatsStruct()
        _check(load().prismq_server_stats_get(self.h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in st._fields_}
