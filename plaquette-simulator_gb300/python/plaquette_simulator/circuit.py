"""Compiled circuits on one ``CliffordState`` (C ABI ``ps_circuit_*``).

``CompiledCircuit(circuit, state, fused=True, graph=True)`` binds a
``circuits.Circuit`` to a state.  ``fused=False`` is the plain form (one
kernel launch per op, the reference's CliffordCircuit::Execute structure,
CliffordCircuit.hpp:131-135); ``fused=True`` applies every run of gates
between measurement phases in one tableau pass.  ``graph=True`` captures the
plan once in a CUDA graph.  ``shared_xz=True`` (the default) lets fused runs
from |0...0> of a circuit without per-shot conditional gates share the x / z
bits of all shots and run only a sign program per shot-word (bit-identical;
the final x / z bits are written to every shot); ``shared_xz=False`` updates
every shot's tableau in every run.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check
from .circuits import Circuit
from .simulator import CliffordState, _ptr


class CircuitOptions(C.Structure):
    _fields_ = [("mode", C.c_int32), ("use_graph", C.c_int32), ("seg_rows", C.c_int32),
                ("seg_words", C.c_int32), ("seg_threads", C.c_int32), ("meas_words", C.c_int32),
                ("seg_resident", C.c_int32), ("per_shot_xz", C.c_int32), ("frame_warps", C.c_int32),
                ("bcast_ctas", C.c_int32)]


class CircuitStats(C.Structure):
    _fields_ = [("num_ops", C.c_uint64), ("num_gates", C.c_uint64), ("num_measurements", C.c_uint64),
                ("num_channels", C.c_uint64), ("num_events", C.c_uint64), ("num_segments", C.c_uint64),
                ("num_measure_phases", C.c_uint64), ("launches_per_run", C.c_uint64),
                ("first_record", C.c_uint64), ("segment_bytes", C.c_double), ("seg_rows", C.c_int32),
                ("seg_words", C.c_int32), ("seg_threads", C.c_int32), ("meas_words", C.c_int32),
                ("resident_segments", C.c_int32), ("shared_xz", C.c_int32),
                ("frame_warps", C.c_int32), ("bcast_ctas", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CompiledCircuit:
    def __init__(self, circuit: Circuit, state: CliffordState, fused: bool = True, graph: bool = True,
                 seg_rows: int = 0, seg_words: int = 0, seg_threads: int = 0, meas_words: int = 0,
                 resident: bool = False, word_vector: bool = False, shared_xz: bool = True,
                 frame_warps: int = 0, bcast_ctas: int = 0):
        if circuit.num_qubits != state.get_num_qubits():
            raise ValueError("circuit and state have different qubit counts")
        self._L = _lib.load()
        self.state = state
        self.circuit = circuit
        self._ops = np.ascontiguousarray(circuit.op_array(), dtype=np.int32)
        self._params = np.ascontiguousarray(circuit.param_array(), dtype=np.float32)
        opts = CircuitOptions(1 if fused else 0, 1 if graph else 0, seg_rows, seg_words, seg_threads, meas_words,
                              2 if word_vector else (1 if resident else 0), 0 if shared_xz else 1, frame_warps,
                              bcast_ctas)
        h = C.c_void_p()
        check(self._L.ps_circuit_compile(state.handle, _ptr(self._ops), len(self._ops), _ptr(self._params),
                                         len(self._params), C.byref(opts), C.byref(h)))
        self._h = h
        self.stats = self.get_stats()

    @classmethod
    def _borrowed(cls, handle, circuit: Circuit, state: CliffordState) -> "CompiledCircuit":
        """A view of a circuit owned by someone else (a batch job)."""
        self = cls.__new__(cls)
        self._L = _lib.load()
        self.state, self.circuit = state, circuit
        self._h = None
        self._view = C.c_void_p(handle)
        self.stats = self.get_stats()
        return self

    @property
    def _handle(self):
        return self._h if self._h is not None else self._view

    def autotune(self) -> dict:
        """Time tile shapes on this circuit's state and keep the fastest
        (ps_circuit_autotune); returns the chosen options and the tuning time."""
        o = CircuitOptions()
        ms = C.c_double()
        check(self._L.ps_circuit_autotune(self._handle, C.byref(o), C.byref(ms)))
        self.stats = self.get_stats()
        return {"seg_rows": o.seg_rows, "seg_words": o.seg_words, "seg_threads": o.seg_threads,
                "meas_words": o.meas_words, "tune_ms": ms.value}

    def get_stats(self) -> dict:
        st = CircuitStats()
        check(self._L.ps_circuit_get_stats(self._handle, C.byref(st)))
        return st.as_dict()

    @property
    def first_record(self) -> int:
        return int(self.stats["first_record"])

    def set_forced(self, forced_all: Optional[np.ndarray]) -> None:
        """Forced draws: one row of ceil(batch/8) packed bytes per M / R."""
        if forced_all is None:
            check(self._L.ps_circuit_set_forced(self._handle, None))
            return
        f = np.ascontiguousarray(forced_all, dtype=np.uint8)
        nb = (self.state.get_batch_size() + 7) // 8
        if f.shape != (self.stats["num_measurements"], nb):
            raise ValueError(f"forced draws must have shape ({self.stats['num_measurements']}, {nb})")
        check(self._L.ps_circuit_set_forced(self._handle, _ptr(f)))

    def run(self, reset: bool = False) -> None:
        """Enqueue one run on the state's stream (asynchronous)."""
        check(self._L.ps_circuit_run(self._handle, 1 if reset else 0))

    PROFILE_KINDS = ("init", "channel_sample", "segment", "measure", "gate", "channel", "sign_program",
                     "xz_broadcast")

    def profile(self, reset: bool = True) -> dict:
        """Device time per kernel kind of one run (CUDA events around every
        launch; the plan is enqueued launch by launch)."""
        class _Prof(C.Structure):
            _fields_ = [("ms", C.c_double * len(CompiledCircuit.PROFILE_KINDS)),
                        ("launches", C.c_uint64 * len(CompiledCircuit.PROFILE_KINDS))]
        p = _Prof()
        check(self._L.ps_circuit_profile(self._handle, 1 if reset else 0, C.byref(p)))
        return {k: {"ms": p.ms[i], "launches": int(p.launches[i])} for i, k in enumerate(self.PROFILE_KINDS)}

    def measure_stats(self, reset: bool = True):
        """(random_branch, rows_multiplied) per measurement of one run, for
        the first 64 shots."""
        nm = int(self.stats["num_measurements"])
        rnd = np.zeros(max(nm, 1), np.int32)
        rows = np.zeros(max(nm, 1), np.int32)
        check(self._L.ps_circuit_measure_stats(self._handle, 1 if reset else 0, _ptr(rnd), _ptr(rows)))
        return rnd[:nm], rows[:nm]

    def measure_bytes(self, reset: bool = True) -> float:
        """Algorithmic HBM bytes of all measurements of one run, per shot bit:
        deterministic  n + k'*2n + (2n+1);  random  2n + 2k(2n+1) + 3(2n+1)."""
        rnd, rows = self.measure_stats(reset)
        n = self.state.get_num_qubits()
        B8 = self.state.get_batch_size() / 8.0
        det_bits = n + rows * 2 * n + (2 * n + 1)
        rnd_bits = 2 * n + 2 * rows * (2 * n + 1) + 3 * (2 * n + 1)
        return float(np.where(rnd > 0, rnd_bits, det_bits).sum() * B8)

    def copy_records_words(self, results: Optional[np.ndarray] = None, determined: Optional[np.ndarray] = None):
        """Copy every record of the circuit to host arrays of shape
        [num_measurements, words] uint64 (pinned buffers give async speed)."""
        words = C.c_uint64()
        check(self._L.ps_circuit_copy_records(self._handle, _ptr(results), _ptr(determined), C.byref(words)))
        return words.value

    def copy_records_async(self, results: np.ndarray, determined: np.ndarray, stream: Optional[int] = None) -> None:
        """Enqueue the copy of the latest run's records into pinned host arrays
        [num_measurements, words] uint64 and return at once; the arrays hold
        them after wait_records().  The next run of this circuit waits on the
        device for the copy; two compiled copies of one circuit, run in turn,
        overlap one run's copy with the next run."""
        check(self._L.ps_circuit_copy_records_async(self._handle, _ptr(results), _ptr(determined), stream))

    def wait_records(self) -> None:
        check(self._L.ps_circuit_wait_records(self._handle))

    def detectors(self, definitions) -> np.ndarray:
        """XOR of measurement records per detector, computed on the device:
        definitions is a list of lists of measurement indices (program
        order); returns [len(definitions), words] uint64 (bit s of word k =
        shot 64k+s)."""
        defs = [list(d) for d in definitions]
        off = np.zeros(len(defs) + 1, np.uint64)
        off[1:] = np.cumsum([len(d) for d in defs])
        idx = np.ascontiguousarray(np.concatenate([np.asarray(d, np.uint32) for d in defs])
                                   if defs and off[-1] else np.zeros(1, np.uint32), dtype=np.uint32)
        w = ((self.state.get_batch_size() + 63) // 64 + 1) & ~1
        out = np.zeros((len(defs), w), np.uint64)
        if defs:
            check(self._L.ps_circuit_detectors(self._handle, _ptr(idx), _ptr(off), len(defs), _ptr(out)))
        return out

    def records(self):
        """(results, determined) int32 arrays [num_measurements, batch]."""
        self.state.synchronize()
        first, nm = self.first_record, int(self.stats["num_measurements"])
        res = np.empty((nm, self.state.get_batch_size()), np.int32)
        det = np.empty_like(res)
        for k in range(nm):
            res[k], det[k] = self.state.record(first + k)
        return res, det

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and not _lib.exiting():
            try:
                self._L.ps_circuit_destroy(h)
            except Exception:
                pass
            self._h = None


def compile_cache_stats() -> dict:
    """Hits, misses and entries of the process-wide compile cache
    (ps_compile_cache_stats): a circuit compiled again reuses the
    shot-independent host work of its first compile."""
    L = _lib.load()
    h, m, e = C.c_uint64(), C.c_uint64(), C.c_uint64()
    check(L.ps_compile_cache_stats(C.byref(h), C.byref(m), C.byref(e)))
    return {"hits": h.value, "misses": m.value, "entries": e.value}


def compile_cache_clear() -> None:
    check(_lib.load().ps_compile_cache_clear())
