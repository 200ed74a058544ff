"""flow_gb300 -- GB300 (sm_103a) kernel set for the flow 2-D Lagrangian-Eulerian
hydrodynamics mini-app, driven from Python through its C ABI.

The compute lives in ``libflow_gb300.so`` (hand-written CUDA, built by
``flow_gb300.build``); this module only binds the C ABI of
``include/flow_gb300.h`` with ctypes and uses PyTorch for device memory and
streams.  There is no CPU fallback: every call fails loudly when the library or
a GPU is missing.

Layout and names follow the reference host driver (main.c:18-91): a ``Mesh``
with padded sizes (pad = 2), cell arrays of ``nx*ny`` doubles and face/flux
arrays of ``(nx+1)*(ny+1)`` doubles.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .problems import PAD, C_T, Problem  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflow_gb300.so")

GB300_OK = 0
GB300_ERR_CUDA = 1
GB300_ERR_ARG = 2
GB300_ERR_TIMEOUT = 3
GB300_ERR_STATE = 4
MODE_EXACT = 0
MODE_FUSED = 1
MODE_FUSED_LAG = 2

_dp = ctypes.POINTER(ctypes.c_double)


class Mesh(ctypes.Structure):
    """ctypes mirror of ``Mesh`` in include/flow_mesh.h."""

    _fields_ = [
        ("global_nx", ctypes.c_int), ("global_ny", ctypes.c_int),
        ("local_nx", ctypes.c_int), ("local_ny", ctypes.c_int),
        ("pad", ctypes.c_int), ("x_off", ctypes.c_int), ("y_off", ctypes.c_int),
        ("rank", ctypes.c_int), ("nranks", ctypes.c_int), ("niters", ctypes.c_int),
        ("neighbours", ctypes.c_int * 4),
        ("width", ctypes.c_double), ("height", ctypes.c_double),
        ("max_dt", ctypes.c_double), ("sim_end", ctypes.c_double),
        ("dt", ctypes.c_double), ("dt_h", ctypes.c_double),
        ("edgex", _dp), ("edgey", _dp), ("edgedx", _dp), ("edgedy", _dp),
        ("celldx", _dp), ("celldy", _dp),
    ]


class FlowError(RuntimeError):
    pass


_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    """Loads the kernel set; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise FlowError(f"{LIB_PATH} is missing: run `python -m flow_gb300.build` "
                            "(the GB300 kernel set has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH, mode=os.RTLD_LOCAL)
        _declare(L)
        _lib = L
        return L


def _declare(L: ctypes.CDLL) -> None:
    I, D, P, M, V = ctypes.c_int, ctypes.c_double, _dp, ctypes.POINTER(Mesh), ctypes.c_void_p
    void = {
        "solve_hydro_2d": [M, I] + [P] * 17,
        "set_timestep": [I, I, P, P, P, P, M, P, I, P, P],
        "print_conservation": [I, I, P, P, P, M],
        "equation_of_state": [I, I, P, P, P],
        "pressure_acceleration": [I, I, M, D, P, P, P, P, P, P, P, P, P, P],
        "artificial_viscosity": [I, I, M, D, P, P, P, P, P, P, P, P, P, P, P],
        "shock_heating_and_work": [I, I, M, D, P, P, P, P, P, P, P, P, P],
        "advect_mass_and_energy": [I, I, M, I, D, D] + [P] * 13,
        "x_mass_and_energy_flux": [I, I, I, M, D, D] + [P] * 10,
        "y_mass_and_energy_flux": [I, I, I, M, D, D] + [P] * 10,
        "advect_momentum": [I, I, I, M, D, D] + [P] * 15,
        "momentum_x_flux_in_x": [I, I, M, D, P, P, P, P, P, P],
        "momentum_x_flux_in_y": [I, I, M, D, P, P, P, P, P, P, P],
        "momentum_y_flux_in_x": [I, I, M, D, P, P, P, P, P, P, P],
        "momentum_y_flux_in_y": [I, I, M, D, P, P, P, P, P, P],
        "handle_boundary_2d": [I, I, M, P, I, I],
    }
    for name, args in void.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, None
    status = {
        "gb300_last_error": [],
        "gb300_set_stream": [V],
        "gb300_set_mode": [I],
        "gb300_set_lagrangian_rows": [I],
        "gb300_get_mode": [],
        "gb300_set_verbose": [I],
        "gb300_synchronize": [],
        "gb300_state_changed": [],
        "gb300_solve_hydro_2d": [M, I] + [P] * 17,
        "gb300_conservation": [I, I, I, P, P, P, P, I],
        "gb300_conservation_noalloc": [I, I, I, P, P, P],
        "gb300_fill_boxes": [I, I, P, P, P, I, P, P],
        "gb300_profile_enable": [I],
        "gb300_profile_reset": [],
        "gb300_profile_count": [],
        "gb300_profile_entry": [I, ctypes.c_char_p, I, ctypes.POINTER(ctypes.c_longlong), P],
        "gb300_measure_fp64_fma_rate": [P],
        "gb300_check_fp64_helpers": [ctypes.c_longlong, ctypes.c_ulonglong,
                                     ctypes.POINTER(ctypes.c_longlong),
                                     ctypes.POINTER(ctypes.c_longlong), P],
        "gb300_mixed_prepare": [M, P, P, V, ctypes.c_size_t, P, I],
        "gb300_mixed_solve": [M, I, P, P, V, V, V, ctypes.c_size_t, P],
    }
    for name, args in status.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, ctypes.c_int
    L.gb300_last_error_message.argtypes, L.gb300_last_error_message.restype = [], ctypes.c_char_p
    L.gb300_clear_error.argtypes, L.gb300_clear_error.restype = [], None
    L.gb300_get_stream.argtypes, L.gb300_get_stream.restype = [], ctypes.c_void_p
    L.gb300_launch_count.argtypes, L.gb300_launch_count.restype = [], ctypes.c_ulonglong
    L.gb300_mixed_workspace_bytes.argtypes = [I, I]
    L.gb300_mixed_workspace_bytes.restype = ctypes.c_size_t
    L.gb300_mixed_workspace_offset.argtypes = [I, I, I]
    L.gb300_mixed_workspace_offset.restype = ctypes.c_size_t
    IP = ctypes.POINTER(ctypes.c_int)
    batch = {
        "gb300_batch_create": [I, IP, IP, P, P, I, ctypes.POINTER(V)],
        "gb300_batch_bind": [V, V, ctypes.c_size_t],
        "gb300_batch_set_state": [V, I, P, P, D],
        "gb300_batch_fill_boxes": [V, I, P, I, D],
        "gb300_batch_set_tuning": [V, I, I, I],
        "gb300_batch_get_tuning": [V, IP, IP, IP, IP],
        "gb300_batch_step": [V, I, I],
        "gb300_batch_status": [V],
        "gb300_batch_set_spin_limit": [V, ctypes.c_longlong],
        "gb300_batch_set_schedule": [V, I],
        "gb300_batch_get_schedule": [V],
        "gb300_batch_get_state": [V, I, P, P, P, P],
    }
    for name, args in batch.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, ctypes.c_int
    L.gb300_batch_pool_bytes.argtypes, L.gb300_batch_pool_bytes.restype = [V], ctypes.c_size_t
    L.gb300_batch_cells.argtypes, L.gb300_batch_cells.restype = [V], ctypes.c_longlong
    L.gb300_batch_destroy.argtypes, L.gb300_batch_destroy.restype = [V], None
    L.gb300_set_verbose(0)


def check() -> None:
    """Raises FlowError if the last C ABI call recorded an error."""
    L = lib()
    code = L.gb300_last_error()
    if code != GB300_OK:
        msg = L.gb300_last_error_message().decode()
        L.gb300_clear_error()
        raise FlowError(f"flow_gb300 error {code}: {msg}")


def set_stream(stream) -> None:
    """Routes every launch to a torch.cuda.Stream (or a raw handle)."""
    handle = getattr(stream, "cuda_stream", stream)
    lib().gb300_set_stream(ctypes.c_void_p(int(handle) if handle else None))


def set_mode(mode: int) -> None:
    if lib().gb300_set_mode(mode) != GB300_OK:
        check()


def boxes_array(boxes) -> "ctypes.Array":
    """(density, energy, xpos, ypos, width, height) boxes as a flat C array."""
    flat = [float(v) for b in boxes for v in b]
    return (ctypes.c_double * max(1, len(flat)))(*flat)


def dptr(t) -> "ctypes._Pointer":
    """ctypes double* of a CUDA torch tensor."""
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), _dp)


def vptr(t) -> ctypes.c_void_p:
    """void* of a CUDA torch tensor."""
    return ctypes.c_void_p(t.data_ptr())


from .sim import DeviceSim, MixedSim  # noqa: E402,F401
from .batch import Batch  # noqa: E402,F401
