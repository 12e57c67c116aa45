"""ctypes binding of the C ABI (``include/cem.h``) of the CUDA library.

The library is built in-tree (``casmcode_clexmonte_gb300/_build``) by
``casmcode_clexmonte_gb300.build``. There is no CPU fallback: if the library
is missing, or no CUDA device is present, calls raise.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

CEM_OK = 0
CEM_STOPPED = 5  # cem_synchronize: the run was stopped early (not an error)
CEM_SEMIGRAND_CANONICAL = 0
CEM_CANONICAL = 1

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_hp = C.POINTER(C.c_int16)


class SystemDesc(C.Structure):
    _fields_ = [
        ("n_sublat", C.c_int), ("n_occ", C.c_int), ("n_funcs", C.c_int), ("n_orbits", C.c_int),
        ("orbit_size", _ip), ("orbit_func_begin", _ip), ("orbit_n_funcs", _ip),
        ("weights", _dp),
        ("n_flower", C.c_int), ("flower_sublat", _ip), ("flower_orbit", _ip),
        ("flower_partner_sublat", _ip), ("flower_partner_du", _ip), ("flower_lut", _hp),
        ("n_owned", C.c_int), ("owned_sublat", _ip), ("owned_orbit", _ip),
        ("owned_partner_sublat", _ip), ("owned_partner_du", _ip), ("owned_lut", _hp),
        ("n_neighbour", _ip), ("neighbour_sublat", _ip), ("neighbour_du", _ip),
        ("param_RT", _dp),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("n_samples", C.c_double), ("mean_potential", C.c_double), ("var_potential", C.c_double),
        ("mean_formation", C.c_double), ("mean_comp", C.c_double * 3),
        ("cov_comp", C.c_double * 9), ("cov_e_comp", C.c_double * 3), ("energy", C.c_double),
        ("n_proposed", C.c_int64), ("n_accepted", C.c_int64), ("passes", C.c_int64),
    ]


# every entry point of include/cem.h
EXPORTS = [
    "cem_last_error", "cem_device_info", "cem_system_create", "cem_system_destroy",
    "cem_replicas_create", "cem_replicas_create_supercells", "cem_supercell_hnf", "cem_replicas_destroy", "cem_n_sites", "cem_set_conditions",
    "cem_set_seed", "cem_set_occupation", "cem_get_occupation", "cem_set_occupation_all",
    "cem_get_occupation_all", "cem_host_alloc", "cem_host_free", "cem_energy",
    "cem_delta_energy", "cem_replay", "cem_enforce_composition", "cem_nfold_run", "cem_run", "cem_get_stats", "cem_get_samples",
    "cem_reset_stats", "cem_synchronize", "cem_request_stop", "cem_last_kernel_ms", "cem_smem_bandwidth",
    "cem_set_option", "cem_get_option", "cem_autotune", "cem_step_async", "cem_delta_energy_noalloc",
    "cem_mlp_info", "cem_mlp_create", "cem_mlp_destroy", "cem_mlp_get_params",
    "cem_mlp_set_params", "cem_mlp_forward", "cem_mlp_forward_tc",
    "cem_mlp_gradient", "cem_mlp_train",
    "cem_learned_features", "cem_learned_run", "cem_learned_group_run", "cem_learned_samples",
    "cem_get_order_samples",
    "cem_state_bytes", "cem_get_state", "cem_set_state",
]

_lib = None


def load(path: str = LIB):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"CUDA library {path} is missing: run `python -m casmcode_clexmonte_gb300.build`"
        )
    L = C.CDLL(path)
    P = C.c_void_p
    vp = C.c_void_p
    L.cem_last_error.restype = C.c_char_p
    L.cem_device_info.argtypes = [C.c_char_p, C.c_int, _ip, _ip, _ip]
    L.cem_system_create.argtypes = [C.POINTER(SystemDesc), C.POINTER(P)]
    L.cem_system_destroy.argtypes = [P]
    L.cem_replicas_create.argtypes = [P, C.c_int, _ip, C.c_int, C.POINTER(P)]
    L.cem_replicas_create_supercells.argtypes = [P, C.c_int, vp, C.c_int, C.POINTER(P)]
    L.cem_supercell_hnf.argtypes = [vp, vp]
    L.cem_replicas_destroy.argtypes = [P]
    L.cem_n_sites.argtypes = [P, C.c_int, C.POINTER(C.c_int64)]
    L.cem_set_conditions.argtypes = [P, C.c_int, C.c_double, _dp]
    L.cem_set_seed.argtypes = [P, C.c_int, C.c_uint64]
    L.cem_set_occupation.argtypes = [P, C.c_int, vp]
    L.cem_get_occupation.argtypes = [P, C.c_int, vp]
    L.cem_set_occupation_all.argtypes = [P, vp]
    L.cem_get_occupation_all.argtypes = [P, vp]
    L.cem_host_alloc.argtypes = [C.c_int64, C.POINTER(vp)]
    L.cem_host_free.argtypes = [vp]
    L.cem_energy.argtypes = [P, C.c_int, _dp, vp]
    L.cem_delta_energy.argtypes = [P, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int, vp, vp]
    L.cem_replay.argtypes = [P, C.c_int, C.c_uint64, C.c_int64, vp, vp, vp,
                             C.POINTER(C.c_int64), C.POINTER(C.c_uint64)]
    L.cem_enforce_composition.argtypes = [P, _dp, C.c_uint64, C.POINTER(C.c_int64)]
    L.cem_nfold_run.argtypes = [P, C.c_int64, C.c_int64, C.c_int64, vp, vp, vp]
    L.cem_run.argtypes = [P, C.c_int64, C.c_int64, C.c_int]
    L.cem_autotune.argtypes = [P, C.c_int64, C.POINTER(C.c_double)]
    L.cem_step_async.argtypes = [P, vp, vp, C.c_int64]
    L.cem_get_stats.argtypes = [P, C.c_int, C.POINTER(Stats)]
    L.cem_get_samples.argtypes = [P, C.c_int, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.cem_reset_stats.argtypes = [P]
    L.cem_synchronize.argtypes = [P]
    L.cem_last_kernel_ms.argtypes = [P, _dp]
    L.cem_smem_bandwidth.argtypes = [_dp]
    L.cem_set_option.argtypes = [P, C.c_char_p, C.c_int64]
    L.cem_mlp_info.argtypes = [_ip, _ip, _ip]
    L.cem_state_bytes.argtypes = [P, C.POINTER(C.c_int64)]
    L.cem_get_state.argtypes = [P, C.c_int, vp, vp]
    L.cem_set_state.argtypes = [P, C.c_int, vp, vp]
    L.cem_get_order_samples.argtypes = [P, C.c_int, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.cem_mlp_create.argtypes = [C.c_uint64, C.POINTER(P)]
    L.cem_mlp_destroy.argtypes = [P]
    L.cem_mlp_get_params.argtypes = [P, vp]
    L.cem_mlp_set_params.argtypes = [P, vp]
    L.cem_mlp_forward.argtypes = [P, C.c_int64, vp, vp]
    L.cem_mlp_forward_tc.argtypes = [P, C.c_int64, vp, vp]
    L.cem_mlp_gradient.argtypes = [P, C.c_int64, vp, vp, vp, C.POINTER(C.c_double)]
    L.cem_mlp_train.argtypes = [P, C.c_int64, vp, vp, C.c_int, C.c_int, C.c_float, C.c_uint64, vp]
    L.cem_learned_features.argtypes = [P, C.c_int, vp, vp]
    L.cem_learned_run.argtypes = [P, P, C.c_int64, C.c_int64, C.c_int]
    L.cem_learned_group_run.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64,
                                        C.c_int]
    L.cem_learned_samples.argtypes = [P, C.c_int, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.cem_get_option.argtypes = [P, C.c_char_p, C.POINTER(C.c_int64)]
    _lib = L
    return L


def check(rc: int):
    if rc != CEM_OK:
        raise RuntimeError(f"cem error {rc}: {load().cem_last_error().decode()}")


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def iptr(a):
    return a.ctypes.data_as(_ip)


def dptr(a):
    return a.ctypes.data_as(_dp)


def hptr(a):
    return a.ctypes.data_as(_hp)


def make_desc(arrs: dict):
    """Build a SystemDesc from ``system.system_arrays``; returns (desc, keepalive)."""
    keep = {k: np.ascontiguousarray(v) for k, v in arrs.items() if isinstance(v, np.ndarray)}
    d = SystemDesc()
    for k in ("n_sublat", "n_occ", "n_funcs", "n_orbits", "n_flower", "n_owned"):
        setattr(d, k, int(arrs[k]))
    for k, v in keep.items():
        if v.dtype == np.int32:
            setattr(d, k, iptr(v))
        elif v.dtype == np.float64:
            setattr(d, k, dptr(v))
        elif v.dtype == np.int16:
            setattr(d, k, hptr(v))
    return d, keep
