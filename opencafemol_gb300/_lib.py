"""ctypes binding of ``libocm_gb300.so`` (the C ABI declared in include/ocm.h).

The library is built in-tree by ``opencafemol_gb300.build.build()``.  It is
mapped on the first call into it (so that the numpy-only parts of the
package, e.g. the seeded system generators, can be used by processes that
must not load the engine).  There is no fallback: if the library is missing
or does not load, that first call raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libocm_gb300.so"

OCM_MAX_GROUPS = 32

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "NEIGHBOR_OVERFLOW",
    5: "STATE", 6: "UNSUPPORTED", 7: "NONFINITE", 8: "TIMEOUT",
}


class OCMError(RuntimeError):
    """Error raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class ContextStats(C.Structure):
    _fields_ = [("steps_done", C.c_int64), ("list_builds", C.c_int64), ("tiles", C.c_int64),
                ("masked_tiles", C.c_int64), ("rebuild_interval", C.c_int32),
                ("reordered", C.c_int32), ("skin", C.c_double), ("max_cutoff", C.c_double),
                ("tile_cutoff", C.c_double), ("charged_pairs", C.c_int64), ("charged_split", C.c_int32),
                ("one_system", C.c_int32)]


_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)
_CP = C.c_char_p

# name -> (restype, argtypes)
SIGNATURES = {
    "ocm_last_error": (C.c_char_p, []),
    "ocm_abi_version": (C.c_int, []),
    "ocm_device_count": (C.c_int, []),
    "ocm_fla_table": (C.c_int, [_CP, _DP, _DP]),
    "ocm_fld_table": (C.c_int, [_CP, _DP]),
    "ocm_fld_table_key": (C.c_int, [C.c_int, C.c_char_p, C.c_int64]),
    "ocm_topology_create": (C.c_int, [C.c_int64, C.POINTER(_P)]),
    "ocm_topology_destroy": (None, [_P]),
    "ocm_topology_add_edges": (C.c_int, [_P, C.c_int64, _I64P, _CP]),
    "ocm_topology_make_molecule": (C.c_int, [_P, _CP]),
    "ocm_topology_ignore_list_within_edge": (C.c_int, [_P, C.c_int64, _CP, _I64P, C.c_int64, _I64P]),
    "ocm_topology_ignore_list_within_molecule": (C.c_int, [_P, _I64P, C.c_int64, _I64P]),
    "ocm_system_create": (C.c_int, [C.c_int64, _DP, C.POINTER(_P)]),
    "ocm_system_destroy": (None, [_P]),
    "ocm_system_set_pbc": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    "ocm_system_num_particles": (C.c_int64, [_P]),
    "ocm_system_num_groups": (C.c_int, [_P]),
    "ocm_system_group_name": (C.c_int, [_P, C.c_int, C.c_char_p, C.c_int64]),
    "ocm_system_describe": (C.c_int, [_P, C.c_char_p, C.c_int64, _I64P]),
    "ocm_add_harmonic_bond": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, C.c_int, _I32P]),
    "ocm_add_go_contact": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, C.c_int, _I32P]),
    "ocm_add_gaussian_bond": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, _DP, C.c_int, _I32P]),
    "ocm_add_gaussian_dihedral": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, _DP, C.c_int, _I32P]),
    "ocm_add_flexible_local_angle": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, _CP, C.c_int, _I32P]),
    "ocm_add_flexible_local_dihedral": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, _CP, C.c_int, _I32P]),
    "ocm_add_excluded_volume": (C.c_int, [_P, C.c_double, C.c_double, _DP, C.c_int64, _I64P, C.c_int,
                                          C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_debye_huckel": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, _DP, C.c_int64, _I64P,
                                       C.c_int, C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_lennard_jones_repulsive": (C.c_int, [_P, C.c_double, _DP, _DP, C.c_int64, _I64P, C.c_int,
                                                  C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_lennard_jones_attractive": (C.c_int, [_P, C.c_double, _DP, _DP, C.c_int64, _I64P, C.c_int,
                                                   C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_weeks_chandler_andersen": (C.c_int, [_P, _DP, _DP, C.c_int64, _I64P, C.c_int,
                                                  C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_uniform_weeks_chandler_andersen": (C.c_int, [_P, C.c_double, C.c_double, C.c_int64, _I64P,
                                                          C.c_int64, _I64P, C.c_int64, _I64P, C.c_int,
                                                          C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_uniform_lennard_jones_attractive": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int64,
                                                           _I64P, C.c_int64, _I64P, C.c_int64, _I64P, C.c_int,
                                                           C.c_int64, _I32P, _I32P, _I32P]),
    "ocm_add_capped_go_contact": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP, C.c_double, C.c_int, _I32P]),
    "ocm_context_minimize": (C.c_int, [_P, C.c_double, C.c_int64, _I64P]),
    "ocm_context_minimize_report": (C.c_int, [_P, _I32P, _DP]),
    "ocm_context_set_engine": (C.c_int, [_P, C.c_int32]),
    "ocm_context_create": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int,
                                     C.POINTER(_P)]),
    "ocm_context_destroy": (None, [_P]),
    "ocm_context_set_positions": (C.c_int, [_P, _DP]),
    "ocm_context_get_positions": (C.c_int, [_P, _DP]),
    "ocm_context_set_velocities": (C.c_int, [_P, _DP]),
    "ocm_context_get_velocities": (C.c_int, [_P, _DP]),
    "ocm_context_set_velocities_to_temperature": (C.c_int, [_P, C.c_double, C.c_int32]),
    "ocm_context_get_state": (C.c_int, [_P, C.c_uint32, _DP, _DP]),
    "ocm_context_get_group_energies": (C.c_int, [_P, _DP]),
    "ocm_context_get_kinetic_energy": (C.c_int, [_P, _DP]),
    "ocm_context_step": (C.c_int, [_P, C.c_int64]),
    "ocm_context_get_stats": (C.c_int, [_P, C.POINTER(ContextStats)]),
    "ocm_context_set_list_options": (C.c_int, [_P, C.c_int32, C.c_double]),
    "ocm_context_list_pairs": (C.c_int, [_P, _I64P, C.c_int64, _I64P]),
    "ocm_context_cluster_order": (C.c_int, [_P, _I64P, C.c_int64, _I64P]),
    "ocm_batch_create": (C.c_int, [C.c_int, C.c_int64, C.c_int64, C.c_int32, C.POINTER(_P)]),
    "ocm_batch_destroy": (None, [_P]),
    "ocm_batch_footprint": (C.c_int64, [_P]),
    "ocm_batch_admit": (C.c_int, [_P, _P, _DP, _DP, C.c_double, C.c_double, C.c_double, C.c_int32,
                                  C.c_int64, _I64P]),
    "ocm_batch_admit_resume": (C.c_int, [_P, _P, _DP, _DP, C.c_double, C.c_double, C.c_double, C.c_int32,
                                         C.c_int64, C.c_int64, _I64P]),
    "ocm_batch_slot_status": (C.c_int, [_P, C.c_int64, _I32P]),
    "ocm_batch_set_balanced": (C.c_int, [_P, C.c_int]),
    "ocm_batch_set_split": (C.c_int, [_P, C.c_int32]),
    "ocm_batch_run": (C.c_int, [_P, C.c_int32, C.c_int]),
    "ocm_batch_finished": (C.c_int, [_P, _I64P, C.c_int64, _I64P]),
    "ocm_batch_get_positions": (C.c_int, [_P, C.c_int64, _DP]),
    "ocm_batch_get_velocities": (C.c_int, [_P, C.c_int64, _DP]),
    "ocm_batch_steps_done": (C.c_int, [_P, C.c_int64, _I64P]),
    "ocm_batch_set_positions_many": (C.c_int, [_P, C.c_int64, _I64P, _DP, _DP]),
    "ocm_batch_get_positions_many": (C.c_int, [_P, C.c_int64, _I64P, _DP]),
    "ocm_batch_get_positions_many_noalloc": (C.c_int, [_P, C.c_int64, _I64P, _DP]),
    "ocm_batch_get_state": (C.c_int, [_P, C.c_int64, C.c_uint32, _DP, _DP]),
    "ocm_batch_retire": (C.c_int, [_P, C.c_int64]),
    "ocm_batch_active": (C.c_int, [_P, _I64P, _I64P]),
    "ocm_batch_last_run_ms": (C.c_int, [_P, _DP]),
    "ocm_batch_set_threads": (C.c_int, [_P, C.c_int32]),
    "ocm_batch_get_threads": (C.c_int, [_P, _I32P]),
    "ocm_batch_set_list_smem": (C.c_int, [_P, C.c_int32]),
    "ocm_batch_slot_stats": (C.c_int, [_P, C.c_int64, _I32P, _I32P]),
}


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class _LazyLib:
    """The ctypes library, loaded on first attribute access."""

    __slots__ = ("_cdll",)

    def __init__(self):
        self._cdll = None

    def loaded(self) -> bool:
        return self._cdll is not None

    def __getattr__(self, name):
        cdll = self._cdll
        if cdll is None:
            cdll = self._cdll = _load()
        return getattr(cdll, name)


lib = _LazyLib()


def check(code: int) -> None:
    if code != 0:
        raise OCMError(code, lib.ocm_last_error().decode(errors="replace"))


def dptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_DP)


def i64ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_I64P)


def i32ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_I32P)


def as_f64(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        arr = arr.reshape(shape)
    return arr


def as_i64(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
    if shape is not None:
        arr = arr.reshape(shape)
    return arr


def as_i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def device_count() -> int:
    return int(lib.ocm_device_count())


def loaded_path() -> str:
    return os.fspath(LIB_PATH)
