"""``CliffordState``: drop-in for the reference's Python binding.

The reference exposes ``plaquette_simulator.CliffordState`` through pybind11
(plaquette_simulator/src/Bindings.cpp:13-31, re-exported by simulator.py:1 and
__init__.py:2).  This class keeps those method names, argument meanings and
return types, and calls the CUDA library through its C ABI
(include/plaquette_gpu.h).  Methods beyond the reference binding are marked.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import PS_E_RANGE, PlaquetteError, check

_vp = C.c_void_p


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_vp)


def _forced_bytes(forced, batch: int) -> Optional[np.ndarray]:
    """Accept per-shot 0/1 values (length batch) or packed LSB-first bytes."""
    if forced is None:
        return None
    a = np.ascontiguousarray(forced, dtype=np.uint8)
    if a.size == batch and a.size != (batch + 7) // 8:
        a = np.packbits(a, bitorder="little")
    if a.size < (batch + 7) // 8:
        raise ValueError("forced bits shorter than the batch")
    return np.ascontiguousarray(a)


class CliffordState:
    """Batched stabilizer tableau on one GPU.

    ``CliffordState(num_qubits, batch_size, seed, init_to_zero)`` as in
    Bindings.cpp:14 (CliffordState.hpp:97-139).  ``seed`` < 0 selects the
    reference's fallback seed.
    """

    def __init__(self, num_qubits: int, batch_size: int, seed: int = -1, init_to_zero: bool = True,
                 _handle=None):
        self._L = _lib.load()
        if _handle is not None:
            self._h = _handle
        else:
            h = C.c_void_p()
            check(self._L.ps_create(num_qubits, batch_size, seed, int(bool(init_to_zero)), C.byref(h)))
            self._h = h
        self._n = self._get_u64("ps_get_num_qubits")
        self._batch = self._get_u64("ps_get_batch_size")

    # -- construction extras (CliffordState.hpp:153-174) -----------------
    @classmethod
    def from_host(cls, x, z, r, num_qubits: int, batch_size: int, seed: int = -1) -> "CliffordState":
        """Host-vector constructor (CliffordState.hpp:153-159)."""
        L = _lib.load()
        xa, za, ra = (np.ascontiguousarray(np.asarray(a).reshape(-1), dtype=np.int32) for a in (x, z, r))
        W = 2 * num_qubits + 1
        if xa.size != batch_size * W * num_qubits or za.size != xa.size or ra.size != batch_size * W:
            raise ValueError("host tableau has the wrong size")
        h = C.c_void_p()
        check(L.ps_create_from_host(_ptr(xa), _ptr(za), _ptr(ra), num_qubits, batch_size, seed, C.byref(h)))
        return cls(num_qubits, batch_size, seed, False, _handle=h)

    def copy(self) -> "CliffordState":
        """Copy constructor (CliffordState.hpp:168-174); records are not copied."""
        h = C.c_void_p()
        check(self._L.ps_clone(self._h, C.byref(h)))
        return CliffordState(self._n, self._batch, _handle=h)

    __copy__ = copy

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and not _lib.exiting():
            try:
                self._L.ps_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def _get_u64(self, fn: str) -> int:
        v = C.c_uint64()
        check(getattr(self._L, fn)(self._h, C.byref(v)))
        return v.value

    # -- reference binding surface (Bindings.cpp:15-31) ------------------
    def get_num_qubits(self) -> int:
        return self._n

    def get_batch_size(self) -> int:
        return self._batch

    def get_seed(self) -> int:
        v = C.c_int64()
        check(self._L.ps_get_seed(self._h, C.byref(v)))
        return v.value

    def reset_clifford_state(self) -> None:
        check(self._L.ps_reset(self._h))

    def get_kokkos_backend(self) -> str:
        return self._L.ps_backend_name().decode()

    def measure_qubit(self, target_qubit: int, bias: float = 0.5, measurement_id: Optional[int] = None,
                      forced=None) -> int:
        """MeasureQubit (CliffordState.hpp:587-623).  ``forced`` (extra):
        per-shot 0/1 draws or packed bits replacing the random draw."""
        out = C.c_uint64()
        f = _forced_bytes(forced, self._batch)
        rid = -1 if measurement_id is None else int(measurement_id)
        try:
            check(self._L.ps_measure(self._h, target_qubit, bias, rid, _ptr(f), C.byref(out)))
        except PlaquetteError as e:
            if e.status == PS_E_RANGE:
                raise RuntimeError(str(e)) from None
            raise
        return out.value

    def get_measurement(self, measurement_id: int, batch_index: int) -> Optional[Tuple[int, int]]:
        """GetMeasurement(id, shot) (CliffordState.hpp:635-648): None where
        the reference returns nullopt."""
        res, det = C.c_int32(), C.c_int32()
        st = self._L.ps_get_measurement(self._h, measurement_id, batch_index, C.byref(res), C.byref(det))
        if st == PS_E_RANGE:
            return None
        check(st)
        return res.value, det.value

    def apply_hadamard_gate(self, q: int) -> None:
        check(self._L.ps_h(self._h, q))

    def apply_phase_gate(self, q: int) -> None:
        check(self._L.ps_s(self._h, q))

    def apply_pauli_x_gate(self, q: int) -> None:
        check(self._L.ps_x(self._h, q))

    def apply_pauli_z_gate(self, q: int) -> None:
        check(self._L.ps_z(self._h, q))

    def apply_control_not_gate(self, control: int, target: int) -> None:
        check(self._L.ps_cx(self._h, control, target))

    def apply_control_phase_gate(self, control: int, target: int) -> None:
        check(self._L.ps_cz(self._h, control, target))

    def device_to_host(self) -> Tuple[List[int], List[int], List[int]]:
        """DeviceToHost (CliffordState.hpp:238-259): flat lists in the
        reference layout x,z [batch][2n+1][n], r [batch][2n+1]."""
        x, z, r = self.device_to_host_numpy()
        return x.reshape(-1).tolist(), z.reshape(-1).tolist(), r.reshape(-1).tolist()

    # -- extras beyond the reference binding -----------------------------
    def apply_pauli_y_gate(self, q: int) -> None:
        """ApplyPauliYGate (CliffordState.hpp:508-510; not bound in Python there)."""
        check(self._L.ps_y(self._h, q))

    def apply_hadamard_gate_with_apply_flag(self, q: int, measurement_id: int) -> None:
        """ApplyHadamardGateWithApplyFlag (CliffordState.hpp:348-356) with the
        flag taken from a measurement record."""
        check(self._L.ps_h_flag(self._h, q, measurement_id))

    def apply_phase_gate_with_apply_flag(self, q: int, measurement_id: int) -> None:
        check(self._L.ps_s_flag(self._h, q, measurement_id))

    def apply_gate_to_qubits(self, code: int, targets: Sequence[int]) -> None:
        t = np.ascontiguousarray(targets, dtype=np.uint64)
        check(self._L.ps_apply_to_qubits(self._h, code, _ptr(t), t.size))

    def measure_qubits(self, targets: Sequence[int], bias: float = 0.5) -> List[int]:
        t = np.ascontiguousarray(targets, dtype=np.uint64)
        first = C.c_uint64()
        check(self._L.ps_measure_qubits(self._h, _ptr(t), t.size, bias, C.byref(first)))
        return list(range(first.value, first.value + t.size))

    def reset_qubit(self, q: int, forced=None) -> int:
        out = C.c_uint64()
        f = _forced_bytes(forced, self._batch)
        check(self._L.ps_reset_qubit(self._h, q, _ptr(f), C.byref(out)))
        return out.value

    def pauli_channel_1(self, q: int, px: float, py: float, pz: float) -> None:
        p = np.asarray([px, py, pz], dtype=np.float32)
        check(self._L.ps_pauli_channel_1(self._h, q, _ptr(p)))

    def pauli_channel_2(self, a: int, b: int, probs: Sequence[float]) -> None:
        p = np.ascontiguousarray(probs, dtype=np.float32)
        if p.size != 15:
            raise ValueError("15 probabilities required")
        check(self._L.ps_pauli_channel_2(self._h, a, b, _ptr(p)))

    def check_sum(self, starting_batch_id: int = 0, ending_batch_id: int = -1) -> int:
        """CheckSum (CliffordState.hpp:327-338)."""
        v = C.c_int64()
        check(self._L.ps_checksum(self._h, starting_batch_id, ending_batch_id, C.byref(v)))
        return v.value

    def device_to_host_numpy(self):
        n, B = self._n, self._batch
        W = 2 * n + 1
        x = np.empty((B, W, n), dtype=np.int32)
        z = np.empty((B, W, n), dtype=np.int32)
        r = np.empty((B, W), dtype=np.int32)
        check(self._L.ps_device_to_host(self._h, _ptr(x), _ptr(z), _ptr(r)))
        return x, z, r

    def host_to_device(self, x, z, r) -> None:
        xa, za, ra = (np.ascontiguousarray(np.asarray(a).reshape(-1), dtype=np.int32) for a in (x, z, r))
        W = 2 * self._n + 1
        if xa.size != self._batch * W * self._n or ra.size != self._batch * W:
            raise ValueError("host tableau has the wrong size")
        check(self._L.ps_host_to_device(self._h, _ptr(xa), _ptr(za), _ptr(ra)))

    def num_records(self) -> int:
        return self._get_u64("ps_num_records")

    def record_bits(self, measurement_id: int) -> Tuple[np.ndarray, np.ndarray]:
        """Packed result / determined bits of one record (LSB-first bytes)."""
        nb = (self._batch + 7) // 8
        res = np.zeros(nb, dtype=np.uint8)
        det = np.zeros(nb, dtype=np.uint8)
        check(self._L.ps_get_record_bits(self._h, measurement_id, _ptr(res), _ptr(det)))
        return res, det

    def record(self, measurement_id: int) -> Tuple[np.ndarray, np.ndarray]:
        """Per-shot int32 (result, determined) arrays of one record."""
        res, det = self.record_bits(measurement_id)
        B = self._batch
        return (np.unpackbits(res, bitorder="little")[:B].astype(np.int32),
                np.unpackbits(det, bitorder="little")[:B].astype(np.int32))

    def event_counter(self) -> int:
        return self._get_u64("ps_get_event_counter")

    def set_event_counter(self, events: int) -> None:
        """The event index the next random op draws with (replays a run)."""
        check(self._L.ps_set_event_counter(self._h, events))

    def set_shot_offset(self, first_shot: int) -> None:
        """This state holds shots [first_shot, first_shot + batch) of a job
        (multiple of 64): draws are keyed by global shot, so a job split over
        several states (one per GPU) reproduces the records of one state."""
        check(self._L.ps_set_shot_offset(self._h, first_shot))

    def shot_offset(self) -> int:
        return self._get_u64("ps_get_shot_offset")

    def tableau_words(self, first_word: int, nwords: int = 1):
        """Packed tableau words of shots [64*first_word, 64*(first_word+nwords)):
        x, z as [2n+1, n, nwords] and r as [2n+1, nwords] uint64."""
        n, W = self.get_num_qubits(), 2 * self.get_num_qubits() + 1
        x = np.zeros((W, n, nwords), np.uint64)
        z = np.zeros_like(x)
        r = np.zeros((W, nwords), np.uint64)
        check(self._L.ps_copy_tableau_words(self._h, first_word, nwords, _ptr(x), _ptr(z), _ptr(r)))
        return x, z, r

    def load_tableau_words(self, first_word: int, x=None, z=None, r=None) -> None:
        """Loads packed words starting at first_word (the layout tableau_words
        returns; a plane left None is kept)."""
        n, W = self.get_num_qubits(), 2 * self.get_num_qubits() + 1
        planes = [None if a is None else np.ascontiguousarray(a, dtype=np.uint64) for a in (x, z, r)]
        nwords = next((a.shape[-1] for a in planes if a is not None), 0)
        for a, shape in zip(planes, ((W, n, nwords), (W, n, nwords), (W, nwords))):
            if a is not None and a.shape != shape:
                raise ValueError(f"packed plane of shape {a.shape}, expected {shape}")
        check(self._L.ps_load_tableau_words(self._h, first_word, nwords,
                                            *(None if a is None else _ptr(a) for a in planes)))

    def snapshot(self) -> dict:
        """Everything a later resume needs: the packed tableau of every shot
        and the event counter (the draws continue from it)."""
        x, z, r = self.tableau_words(0, self.words())
        return {"num_qubits": self.get_num_qubits(), "batch_size": self.get_batch_size(),
                "seed": self.get_seed(), "shot_offset": self.shot_offset(),
                "events": self.event_counter(), "x": x, "z": z, "r": r}

    @classmethod
    def resume(cls, snap: dict) -> "CliffordState":
        """A new state holding a snapshot (records are not part of it)."""
        st = cls(snap["num_qubits"], snap["batch_size"], snap["seed"], True)
        if snap.get("shot_offset", 0):
            st.set_shot_offset(snap["shot_offset"])
        st.load_tableau_words(0, snap["x"], snap["z"], snap["r"])
        st.set_event_counter(snap["events"])
        return st

    def words(self) -> int:
        """64-shot words per tableau column (the batch rounded up to an even
        number of words)."""
        w = C.c_uint64()
        check(self._L.ps_get_device_tableau(self._h, None, None, None, C.byref(w)))
        return w.value

    def synchronize(self) -> None:
        check(self._L.ps_synchronize(self._h))
