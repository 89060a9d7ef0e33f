"""Loader of the CUDA library ``libps_gpu.so`` (C ABI in include/plaquette_gpu.h).

The library is built in-tree by ``plaquette-simulator_gb300/build.py``.  There
is no CPU fallback: if the library is missing or cannot load, importing the
package raises ImportError.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_PATH = os.environ.get("PS_GPU_LIB", os.path.join(PKG_ROOT, "lib", "libps_gpu.so"))

PS_OK, PS_E_ARG, PS_E_RANGE, PS_E_CUDA, PS_E_NOMEM, PS_E_STATE, PS_E_TIMEOUT = range(7)

_u64, _i64, _i32, _f32, _vp = C.c_uint64, C.c_int64, C.c_int32, C.c_float, C.c_void_p
_pp = C.POINTER(C.c_void_p)
_pu64, _pi64, _pi32 = C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)

_SIGS = {
    "ps_last_error": (C.c_char_p, []),
    "ps_backend_name": (C.c_char_p, []),
    "ps_version": (C.c_char_p, []),
    "ps_set_device": (C.c_int, [C.c_int]),
    "ps_device_synchronize": (C.c_int, []),
    "ps_create": (C.c_int, [_u64, _u64, _i64, C.c_int, _pp]),
    "ps_create_from_host": (C.c_int, [_vp, _vp, _vp, _u64, _u64, _i64, _pp]),
    "ps_clone": (C.c_int, [_vp, _pp]),
    "ps_destroy": (C.c_int, [_vp]),
    "ps_get_num_qubits": (C.c_int, [_vp, _pu64]),
    "ps_get_batch_size": (C.c_int, [_vp, _pu64]),
    "ps_get_seed": (C.c_int, [_vp, _pi64]),
    "ps_get_event_counter": (C.c_int, [_vp, _pu64]),
    "ps_set_event_counter": (C.c_int, [_vp, _u64]),
    "ps_set_shot_offset": (C.c_int, [_vp, _u64]),
    "ps_get_shot_offset": (C.c_int, [_vp, _pu64]),
    "ps_reset": (C.c_int, [_vp]),
    "ps_checksum": (C.c_int, [_vp, _i64, _i64, _pi64]),
    "ps_device_to_host": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ps_host_to_device": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ps_h": (C.c_int, [_vp, _u64]),
    "ps_s": (C.c_int, [_vp, _u64]),
    "ps_x": (C.c_int, [_vp, _u64]),
    "ps_y": (C.c_int, [_vp, _u64]),
    "ps_z": (C.c_int, [_vp, _u64]),
    "ps_cx": (C.c_int, [_vp, _u64, _u64]),
    "ps_cz": (C.c_int, [_vp, _u64, _u64]),
    "ps_apply_to_qubits": (C.c_int, [_vp, _i32, _vp, _u64]),
    "ps_h_flag": (C.c_int, [_vp, _u64, _u64]),
    "ps_s_flag": (C.c_int, [_vp, _u64, _u64]),
    "ps_measure": (C.c_int, [_vp, _u64, _f32, _i64, _vp, _pu64]),
    "ps_measure_qubits": (C.c_int, [_vp, _vp, _u64, _f32, _pu64]),
    "ps_get_measurement": (C.c_int, [_vp, _u64, _u64, _pi32, _pi32]),
    "ps_get_record_bits": (C.c_int, [_vp, _u64, _vp, _vp]),
    "ps_num_records": (C.c_int, [_vp, _pu64]),
    "ps_record_qubit": (C.c_int, [_vp, _u64, _pu64]),
    "ps_reset_qubit": (C.c_int, [_vp, _u64, _vp, _pu64]),
    "ps_pauli_channel_1": (C.c_int, [_vp, _u64, _vp]),
    "ps_compile_cache_stats": (C.c_int, [_pu64, _pu64, _pu64]),
    "ps_compile_cache_clear": (C.c_int, []),
    "ps_pauli_channel_2": (C.c_int, [_vp, _u64, _u64, _vp]),
    "ps_pauli_channel_1_noalloc": (C.c_int, [_vp, _u64, _vp]),
    "ps_circuit_compile": (C.c_int, [_vp, _vp, _u64, _vp, _u64, _vp, _pp]),
    "ps_circuit_set_forced": (C.c_int, [_vp, _vp]),
    "ps_circuit_run": (C.c_int, [_vp, C.c_int]),
    "ps_circuit_get_stats": (C.c_int, [_vp, _vp]),
    "ps_circuit_destroy": (C.c_int, [_vp]),
    "ps_circuit_profile": (C.c_int, [_vp, C.c_int, _vp]),
    "ps_circuit_copy_records": (C.c_int, [_vp, _vp, _vp, _pu64]),
    "ps_circuit_copy_records_async": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ps_circuit_wait_records": (C.c_int, [_vp]),
    "ps_circuit_measure_stats": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "ps_circuit_detectors": (C.c_int, [_vp, _vp, _vp, _u64, _vp]),
    "ps_circuit_autotune": (C.c_int, [_vp, _vp, C.POINTER(C.c_double)]),
    "ps_batch_create": (C.c_int, [_vp, _u64, _vp, _pp]),
    "ps_batch_run": (C.c_int, [_vp]),
    "ps_batch_synchronize": (C.c_int, [_vp]),
    "ps_batch_get_stream": (C.c_int, [_vp, _pp]),
    "ps_batch_job": (C.c_int, [_vp, _u64, _pp, _pp]),
    "ps_batch_get_stats": (C.c_int, [_vp, _vp]),
    "ps_batch_destroy": (C.c_int, [_vp]),
    "ps_server_create": (C.c_int, [_vp, _pp]),
    "ps_server_submit": (C.c_int, [_vp, _vp, _pu64]),
    "ps_server_submit_parked": (C.c_int, [_vp, _vp, _vp, _pu64]),
    "ps_server_copy_tableau": (C.c_int, [_vp, _u64, _vp, _vp, _vp, _pu64]),
    "ps_server_wait": (C.c_int, [_vp, _u64, C.c_double, _vp]),
    "ps_server_copy_records": (C.c_int, [_vp, _u64, _vp, _vp]),
    "ps_server_release": (C.c_int, [_vp, _u64]),
    "ps_server_drain": (C.c_int, [_vp, C.c_double]),
    "ps_server_cancel": (C.c_int, [_vp, _u64]),
    "ps_server_get_stats": (C.c_int, [_vp, _vp]),
    "ps_server_now": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "ps_server_destroy": (C.c_int, [_vp]),
    "ps_synchronize": (C.c_int, [_vp]),
    "ps_get_stream": (C.c_int, [_vp, _pp]),
    "ps_get_device_tableau": (C.c_int, [_vp, _pp, _pp, _pp, _pu64]),
    "ps_copy_tableau_words": (C.c_int, [_vp, _u64, _u64, _vp, _vp, _vp]),
    "ps_load_tableau_words": (C.c_int, [_vp, _u64, _u64, _vp, _vp, _vp]),
    "ps_device_to_device": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ps_get_record_device": (C.c_int, [_vp, _u64, _pp, _pp]),
}

_lib = None
_exiting = False


def _mark_exiting():
    global _exiting
    _exiting = True
    if _lib is not None:
        _lib.ps_device_synchronize()  # drain queued kernels before native teardown


# Once the interpreter starts shutting down, finalizers no longer call into
# the library: module teardown order is arbitrary and the process releases
# all device memory on exit anyway.
atexit.register(_mark_exiting)


def exiting() -> bool:
    return _exiting


class PlaquetteError(RuntimeError):
    """Raised for a failed C-ABI call (the reference raises RuntimeError
    from Plaquette::Exception through pybind11)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise ImportError(f"CUDA library not built: {LIB_PATH} is missing "
                          "(run plaquette-simulator_gb300/build.py)")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != PS_OK:
        msg = load().ps_last_error().decode(errors="replace")
        raise PlaquetteError(status, msg)


def exported_symbols():
    """Names the C ABI header declares, parsed from include/plaquette_gpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(PKG_ROOT), "include", "plaquette_gpu.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(ps_[a-z0-9_]+)\s*\(", text)))
