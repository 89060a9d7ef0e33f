"""ctypes front-end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libps_oracle.so`` (the C restatement of the reference's
CliffordState algorithm, ps_oracle.c) and, when it was built here,
``oracle/_ref/libplaquette_ref.so`` (the unmodified reference headers compiled
on the Kokkos-API shim).  Only tests, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference arm import this module; the product
never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libps_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libplaquette_ref.so")

OP_H, OP_S, OP_X, OP_Y, OP_Z, OP_CX, OP_CZ, OP_M, OP_R, OP_PAULI1, OP_PAULI2, OP_H_IF, OP_S_IF = range(13)

_i64, _u64, _i32, _f32, _vp = C.c_int64, C.c_uint64, C.c_int32, C.c_float, C.c_void_p


def build(ref: bool = True) -> None:
    """Compile the oracle (and, if the reference headers exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:  # only where the reference is checked out (REF_SRC, see oracle/Makefile)
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        sig = {
            "ora_create": (_vp, [_i64, _i64, _i64, C.c_int, _i64]),
            "ora_create_from_host": (_vp, [_vp, _vp, _vp, _i64, _i64, _i64, _i64]),
            "ora_clone": (_vp, [_vp]),
            "ora_destroy": (None, [_vp]),
            "ora_num_qubits": (_i64, [_vp]),
            "ora_batch": (_i64, [_vp]),
            "ora_seed": (_i64, [_vp]),
            "ora_events": (_u64, [_vp]),
            "ora_set_threads": (None, [C.c_int]),
            "ora_device_to_host": (None, [_vp, _vp, _vp, _vp]),
            "ora_host_to_device": (None, [_vp, _vp, _vp, _vp]),
            "ora_reset": (None, [_vp]),
            "ora_checksum": (_i64, [_vp, _i64, _i64]),
            "ora_h": (None, [_vp, _i64]),
            "ora_s": (None, [_vp, _i64]),
            "ora_x_gate": (None, [_vp, _i64]),
            "ora_y_gate": (None, [_vp, _i64]),
            "ora_z_gate": (None, [_vp, _i64]),
            "ora_cx": (None, [_vp, _i64, _i64]),
            "ora_cz": (None, [_vp, _i64, _i64]),
            "ora_h_flag": (None, [_vp, _i64, _vp]),
            "ora_s_flag": (None, [_vp, _i64, _vp]),
            "ora_measure": (_i64, [_vp, _i64, _f32, _i64, _vp]),
            "ora_reset_qubit": (_i64, [_vp, _i64, _vp]),
            "ora_num_records": (_i64, [_vp]),
            "ora_get_measurement": (C.c_int, [_vp, _i64, _i64, _vp, _vp]),
            "ora_record_results": (_vp, [_vp, _i64]),
            "ora_record_determined": (_vp, [_vp, _i64]),
            "ora_record_qubit": (_i64, [_vp, _i64]),
            "ora_pauli_channel_1": (None, [_vp, _i64, _vp]),
            "ora_pauli_channel_2": (None, [_vp, _i64, _i64, _vp]),
            "ora_run": (C.c_int, [_vp, _vp, _i64, _vp, _vp]),
            "ora_threshold": (_u64, [C.c_double]),
            "ora_draw_u32": (C.c_uint32, [_i64, _u64, _i64, C.c_uint32]),
            "ora_channel_paulis": (None, [_i64, _u64, _i64, _i64, _vp, C.c_int, _vp]),
            "ora_philox4x32_10": (None, [_vp, _vp, _vp]),
            "ora_row_product_sign": (_i32, [_vp, _i64, _i64, _i64]),
            "ora_row_multiply": (None, [_vp, _i64, _i64, _i64]),
            "ora_measure_determined": (_i32, [_vp, _i64, _i64]),
            "ora_pauli_product_phase": (_i32, [_i32, _i32, _i32, _i32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.isfile(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        sig = {
            "ref_create": (_vp, [_i64, _i64, _i64, C.c_int, _i64]),
            "ref_create_from_host": (_vp, [_vp, _vp, _vp, _i64, _i64, _i64]),
            "ref_destroy": (None, [_vp]),
            "ref_h": (None, [_vp, _i64]),
            "ref_s": (None, [_vp, _i64]),
            "ref_x": (None, [_vp, _i64]),
            "ref_y": (None, [_vp, _i64]),
            "ref_z": (None, [_vp, _i64]),
            "ref_cx": (None, [_vp, _i64, _i64]),
            "ref_cz": (None, [_vp, _i64, _i64]),
            "ref_h_flag": (None, [_vp, _i64, _i64]),
            "ref_s_flag": (None, [_vp, _i64, _i64]),
            "ref_measure": (_i64, [_vp, _i64, _f32, _i64, _vp]),
            "ref_reset_qubit": (_i64, [_vp, _i64, _vp]),
            "ref_get_measurement": (C.c_int, [_vp, _i64, _i64, _vp, _vp]),
            "ref_device_to_host": (None, [_vp, _vp, _vp, _vp]),
            "ref_checksum": (_i64, [_vp, _i64, _i64]),
            "ref_backend": (C.c_char_p, [_vp]),
            "ref_row_product_sign": (_i32, [_vp, _i64, _i64]),
            "ref_row_multiply": (None, [_vp, _i64, _i64]),
            "ref_measure_determined": (_i32, [_vp, _i64]),
            "ref_pauli_product_phase": (_i32, [_i32, _i32, _i32, _i32]),
            "ref_run": (C.c_int, [_vp, _vp, _i64, _vp, _vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _ref = L
    return _ref


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_vp)


def pack_forced(bits: Sequence[int]) -> np.ndarray:
    """Pack per-shot 0/1 values LSB-first into ceil(B/8) bytes."""
    return np.packbits(np.asarray(bits, dtype=np.uint8), bitorder="little")


class _Base:
    """Shared helpers of the two CPU engines (same call surface)."""

    n: int
    batch: int

    def tableau(self):
        n, B = self.n, self.batch
        W = 2 * n + 1
        x = np.empty(B * W * n, dtype=np.int32)
        z = np.empty(B * W * n, dtype=np.int32)
        r = np.empty(B * W, dtype=np.int32)
        self._d2h(x, z, r)
        return x.reshape(B, W, n), z.reshape(B, W, n), r.reshape(B, W)

    def record(self, rid: int):
        res = np.empty(self.batch, dtype=np.int32)
        det = np.empty(self.batch, dtype=np.int32)
        for b in range(self.batch):
            ok, rr, dd = self.get_measurement(rid, b)
            assert ok
            res[b], det[b] = rr, dd
        return res, det


class Oracle(_Base):
    """The C restatement (ps_oracle.c) in the reference's int32 layout."""

    def __init__(self, n: int, batch: int, seed: int = -1, init_zero: bool = True, shot_base: int = 0,
                 host=None):
        L = lib()
        self.n, self.batch = n, batch
        if host is not None:
            x, z, r = (np.ascontiguousarray(a, dtype=np.int32) for a in host)
            self._keep = (x, z, r)
            self.h = L.ora_create_from_host(_ptr(x), _ptr(z), _ptr(r), n, batch, seed, shot_base)
        else:
            self.h = L.ora_create(n, batch, seed, int(init_zero), shot_base)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_destroy(self.h)
            self.h = None

    def h_gate(self, q): lib().ora_h(self.h, q)
    def s_gate(self, q): lib().ora_s(self.h, q)
    def x_gate(self, q): lib().ora_x_gate(self.h, q)
    def y_gate(self, q): lib().ora_y_gate(self.h, q)
    def z_gate(self, q): lib().ora_z_gate(self.h, q)
    def cx(self, c, t): lib().ora_cx(self.h, c, t)
    def cz(self, c, t): lib().ora_cz(self.h, c, t)

    def h_flag(self, q, rec: int):
        lib().ora_h_flag(self.h, q, lib().ora_record_results(self.h, rec))

    def s_flag(self, q, rec: int):
        lib().ora_s_flag(self.h, q, lib().ora_record_results(self.h, rec))

    def measure(self, q, bias=0.5, rid=-1, forced=None):
        f = None if forced is None else np.ascontiguousarray(forced, dtype=np.uint8)
        return lib().ora_measure(self.h, q, bias, rid, _ptr(f))

    def reset_qubit(self, q, forced=None):
        f = None if forced is None else np.ascontiguousarray(forced, dtype=np.uint8)
        return lib().ora_reset_qubit(self.h, q, _ptr(f))

    def pauli_channel_1(self, q, p):
        a = np.asarray(p, dtype=np.float32)
        lib().ora_pauli_channel_1(self.h, q, _ptr(a))

    def pauli_channel_2(self, a, b, p):
        arr = np.asarray(p, dtype=np.float32)
        lib().ora_pauli_channel_2(self.h, a, b, _ptr(arr))

    def get_measurement(self, rid, shot):
        res, det = C.c_int32(), C.c_int32()
        ok = lib().ora_get_measurement(self.h, rid, shot, C.byref(res), C.byref(det))
        return ok == 0, res.value, det.value

    def record(self, rid: int):
        L = lib()
        res = np.ctypeslib.as_array(C.cast(L.ora_record_results(self.h, rid), C.POINTER(C.c_int32)), (self.batch,))
        det = np.ctypeslib.as_array(C.cast(L.ora_record_determined(self.h, rid), C.POINTER(C.c_int32)), (self.batch,))
        return res.copy(), det.copy()

    def num_records(self): return lib().ora_num_records(self.h)
    def checksum(self, s0=0, s1=-1): return lib().ora_checksum(self.h, s0, s1)
    def reset(self): lib().ora_reset(self.h)
    def events(self): return lib().ora_events(self.h)
    def _d2h(self, x, z, r): lib().ora_device_to_host(self.h, _ptr(x), _ptr(z), _ptr(r))

    def run(self, ops: np.ndarray, params: np.ndarray, forced_all: Optional[np.ndarray] = None) -> None:
        ops = np.ascontiguousarray(ops, dtype=np.int32).reshape(-1, 4)
        params = np.ascontiguousarray(params if len(params) else np.zeros(1), dtype=np.float32)
        f = None if forced_all is None else np.ascontiguousarray(forced_all, dtype=np.uint8)
        rc = lib().ora_run(self.h, _ptr(ops), len(ops), _ptr(params), _ptr(f))
        if rc != 0:
            raise ValueError("oracle: bad op in circuit")

    # reference test-only functors
    def row_product_sign(self, shot, i, k): return lib().ora_row_product_sign(self.h, shot, i, k)
    def row_multiply(self, shot, i, k): lib().ora_row_multiply(self.h, shot, i, k)
    def measure_determined(self, shot, q): return lib().ora_measure_determined(self.h, shot, q)


class Reference(_Base):
    """The reference's own CliffordState<int> (unmodified headers on the shim)."""

    def __init__(self, n: int, batch: int, seed: int = -1, init_zero: bool = True, shot_base: int = 0,
                 host=None):
        L = ref_lib()
        self.n, self.batch = n, batch
        if host is not None:
            x, z, r = (np.ascontiguousarray(a, dtype=np.int32) for a in host)
            self.h = L.ref_create_from_host(_ptr(x), _ptr(z), _ptr(r), n, batch, seed)
        else:
            self.h = L.ref_create(n, batch, seed, int(init_zero), shot_base)

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_destroy(self.h)
            self.h = None

    def h_gate(self, q): ref_lib().ref_h(self.h, q)
    def s_gate(self, q): ref_lib().ref_s(self.h, q)
    def x_gate(self, q): ref_lib().ref_x(self.h, q)
    def y_gate(self, q): ref_lib().ref_y(self.h, q)
    def z_gate(self, q): ref_lib().ref_z(self.h, q)
    def cx(self, c, t): ref_lib().ref_cx(self.h, c, t)
    def cz(self, c, t): ref_lib().ref_cz(self.h, c, t)
    def h_flag(self, q, rec): ref_lib().ref_h_flag(self.h, q, rec)
    def s_flag(self, q, rec): ref_lib().ref_s_flag(self.h, q, rec)

    def measure(self, q, bias=0.5, rid=-1, forced=None):
        f = None if forced is None else np.ascontiguousarray(forced, dtype=np.uint8)
        return ref_lib().ref_measure(self.h, q, bias, rid, _ptr(f))

    def reset_qubit(self, q, forced=None):
        f = None if forced is None else np.ascontiguousarray(forced, dtype=np.uint8)
        return ref_lib().ref_reset_qubit(self.h, q, _ptr(f))

    def get_measurement(self, rid, shot):
        res, det = C.c_int32(), C.c_int32()
        ok = ref_lib().ref_get_measurement(self.h, rid, shot, C.byref(res), C.byref(det))
        return ok == 0, res.value, det.value

    def checksum(self, s0=0, s1=-1): return ref_lib().ref_checksum(self.h, s0, s1)
    def backend(self): return ref_lib().ref_backend(self.h).decode()
    def _d2h(self, x, z, r): ref_lib().ref_device_to_host(self.h, _ptr(x), _ptr(z), _ptr(r))

    def run(self, ops, params, forced_all=None):
        ops = np.ascontiguousarray(ops, dtype=np.int32).reshape(-1, 4)
        params = np.ascontiguousarray(params if len(params) else np.zeros(1), dtype=np.float32)
        f = None if forced_all is None else np.ascontiguousarray(forced_all, dtype=np.uint8)
        rc = ref_lib().ref_run(self.h, _ptr(ops), len(ops), _ptr(params), _ptr(f))
        if rc != 0:
            raise ValueError("reference: bad op in circuit")

    def row_product_sign(self, shot, i, k):
        assert shot == 0
        return ref_lib().ref_row_product_sign(self.h, i, k)

    def row_multiply(self, shot, i, k):
        assert shot == 0
        ref_lib().ref_row_multiply(self.h, i, k)

    def measure_determined(self, shot, q):
        assert shot == 0
        return ref_lib().ref_measure_determined(self.h, q)
