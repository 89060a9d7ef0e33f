"""Many sampling jobs at once (C ABI ``ps_batch_*`` and ``ps_server_*``).

``Batch(jobs)`` compiles every job (a ``circuits.Circuit`` with a shot count
and a seed) on its own state; one ``run()`` is one CUDA graph launch holding
every job as an independent branch.  ``Server`` is the request loop: jobs are
submitted as they arrive, admitted against an HBM budget and run
concurrently, one stream per active job; ``wait`` returns the job's latency
and its measurement records.  A job gives the same records in a batch, in a
server mix and alone (``CompiledCircuit`` on a fresh state with the same
seed): the shots of a job only depend on its own seed.

``uneven_surface_jobs`` and ``poisson_arrivals`` draw the job mixes of the
benchmarks (seeded SplitMix64).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check
from .circuits import Circuit, SplitMix64, surface_code_memory


@dataclass
class Job:
    circuit: Circuit
    shots: int
    seed: int
    distance: int = 0
    p: float = 0.0

    @property
    def num_qubits(self) -> int:
        return self.circuit.num_qubits

    def device_bytes(self) -> int:
        """Tableau bytes (x and z planes and r, bit-packed, shots innermost)."""
        n = self.circuit.num_qubits
        w = ((self.shots + 63) // 64 + 1) & ~1
        return (2 * n + 1) * w * 8 * (2 * n + 1)

    def shot_gates(self) -> int:
        g = getattr(self.circuit, "_num_gates", None)
        if g is None:
            g = self.circuit._num_gates = self.circuit.num_gates()
        return g * self.shots


class JobDesc(C.Structure):
    _fields_ = [("ops", C.c_void_p), ("nops", C.c_uint64), ("params", C.c_void_p), ("nparams", C.c_uint64),
                ("num_qubits", C.c_uint64), ("shots", C.c_uint64), ("seed", C.c_int64)]


def _descs(jobs: Sequence[Job]):
    """ctypes descriptors plus the arrays they point into (kept alive)."""
    keep, descs = [], (JobDesc * len(jobs))()
    for i, j in enumerate(jobs):
        ops, par = j.circuit.arrays()
        keep += [ops, par]
        descs[i] = JobDesc(ops.ctypes.data, len(ops), par.ctypes.data if len(par) else None, len(par),
                           j.circuit.num_qubits, j.shots, j.seed)
    return descs, keep


# ------------------------------------------------------------------ batch
class BatchOptions(C.Structure):
    _fields_ = [("autotune", C.c_int32), ("use_graph", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("num_jobs", C.c_uint64), ("shot_gates_per_run", C.c_uint64), ("tableau_bytes", C.c_uint64),
                ("launches_per_run", C.c_uint64), ("compile_ms", C.c_double), ("tune_ms", C.c_double),
                ("table_jobs", C.c_uint64), ("frame_warps", C.c_int32), ("bcast_ctas", C.c_int32)]


class Batch:
    def __init__(self, jobs: Sequence[Job], autotune: bool = True, graph: bool = True):
        self._L = _lib.load()
        self.jobs = list(jobs)
        descs, keep = _descs(self.jobs)
        h = C.c_void_p()
        check(self._L.ps_batch_create(descs, len(self.jobs), C.byref(BatchOptions(int(autotune), int(graph))),
                                      C.byref(h)))
        self._h = h
        st = BatchStats()
        check(self._L.ps_batch_get_stats(self._h, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in st._fields_}

    def run(self) -> None:
        """Enqueue one run of every job (asynchronous)."""
        check(self._L.ps_batch_run(self._h))

    def synchronize(self) -> None:
        check(self._L.ps_batch_synchronize(self._h))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(self._L.ps_batch_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def _job(self, j: int):
        c, s = C.c_void_p(), C.c_void_p()
        check(self._L.ps_batch_job(self._h, j, C.byref(c), C.byref(s)))
        return c, s

    def job_options(self, j: int) -> dict:
        from .circuit import CircuitStats
        c, _ = self._job(j)
        st = CircuitStats()
        check(self._L.ps_circuit_get_stats(c, C.byref(st)))
        return {k: getattr(st, k) for k in ("seg_rows", "seg_words", "seg_threads", "meas_words")}

    def records(self, j: int) -> Tuple[np.ndarray, np.ndarray]:
        """Job j's (results, determined) record words [num_measurements, words]
        uint64 of the last run (waits for the batch)."""
        self.synchronize()
        c, _ = self._job(j)
        nm = self.jobs[j].circuit.num_measurements()
        w = ((self.jobs[j].shots + 63) // 64 + 1) & ~1
        res = np.zeros((nm, w), np.uint64)
        det = np.zeros_like(res)
        words = C.c_uint64()
        check(self._L.ps_circuit_copy_records(c, res.ctypes.data_as(C.c_void_p), det.ctypes.data_as(C.c_void_p),
                                              C.byref(words)))
        return res, det

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value and not _lib.exiting():
            self._L.ps_batch_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------- server
class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_active", C.c_int32), ("autotune", C.c_int32),
                ("hol_wait_s", C.c_double), ("host_pool_bytes", C.c_uint64)]


class JobResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("pad", C.c_int32), ("num_measurements", C.c_uint64),
                ("words", C.c_uint64), ("shot_gates", C.c_uint64), ("device_bytes", C.c_uint64),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("latency_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("queued", C.c_uint64), ("active", C.c_uint64), ("cancelled", C.c_uint64),
                ("tableau_jobs", C.c_uint64),
                ("shot_gates_completed", C.c_uint64),
                ("pool_bytes", C.c_uint64), ("pool_peak_bytes", C.c_uint64), ("p50_latency_s", C.c_double),
                ("p99_latency_s", C.c_double), ("mean_latency_s", C.c_double), ("max_latency_s", C.c_double),
                ("first_submit_s", C.c_double), ("last_done_s", C.c_double)]


class JobPark(C.Structure):
    _fields_ = [("x", C.c_void_p), ("z", C.c_void_p), ("r", C.c_void_p), ("events", C.c_uint64),
                ("keep_tableau", C.c_int32), ("pad", C.c_int32)]


class Server:
    def __init__(self, hbm_budget_bytes: int, max_active: int = 16, autotune: bool = False,
                 hol_wait_s: float = 1.0, host_pool_bytes: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.ps_server_create(C.byref(ServerOptions(hbm_budget_bytes, max_active, int(autotune),
                                                             hol_wait_s, host_pool_bytes)), C.byref(h)))
        self._h = h
        self._jobs = {}

    def now(self) -> float:
        t = C.c_double()
        check(self._L.ps_server_now(self._h, C.byref(t)))
        return t.value

    def submit(self, job: Job, parked: Optional[dict] = None, keep_tableau: bool = False) -> int:
        """Queues a job.  parked: a tableau to start from instead of |0...0>
        (what tableau() gives for an earlier job kept with keep_tableau): the
        circuit then runs without reset and its draws continue from the
        parked event counter."""
        descs, keep = _descs([job])
        jid = C.c_uint64()
        if parked is None and not keep_tableau:
            check(self._L.ps_server_submit(self._h, descs, C.byref(jid)))
        else:
            park = JobPark(None, None, None, 0, int(bool(keep_tableau)), 0)
            if parked is not None:
                arrs = [np.ascontiguousarray(parked[k], dtype=np.uint64) for k in ("x", "z", "r")]
                keep += arrs
                park.x, park.z, park.r = (a.ctypes.data for a in arrs)
                park.events = int(parked["events"])
            check(self._L.ps_server_submit_parked(self._h, descs, C.byref(park), C.byref(jid)))
        self._jobs[jid.value] = job
        return jid.value

    def tableau(self, job_id: int) -> dict:
        """The final packed tableau (x, z [2n+1, n, words], r [2n+1, words]
        uint64) and event counter of a job submitted with keep_tableau."""
        self.wait(job_id)
        job = self._jobs[job_id]
        n, w = job.num_qubits, ((job.shots + 63) // 64 + 1) & ~1
        x = np.zeros((2 * n + 1, n, w), np.uint64)
        z = np.zeros_like(x)
        r = np.zeros((2 * n + 1, w), np.uint64)
        ev = C.c_uint64()
        check(self._L.ps_server_copy_tableau(self._h, job_id, x.ctypes.data_as(C.c_void_p),
                                             z.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p),
                                             C.byref(ev)))
        return {"x": x, "z": z, "r": r, "events": ev.value}

    def wait(self, job_id: int, timeout_s: float = -1.0) -> dict:
        r = JobResult()
        check(self._L.ps_server_wait(self._h, job_id, timeout_s, C.byref(r)))
        return {k: getattr(r, k) for k, _ in r._fields_ if k != "pad"}

    def records(self, job_id: int) -> Tuple[np.ndarray, np.ndarray]:
        r = self.wait(job_id)
        res = np.zeros((r["num_measurements"], r["words"]), np.uint64)
        det = np.zeros_like(res)
        check(self._L.ps_server_copy_records(self._h, job_id, res.ctypes.data_as(C.c_void_p),
                                             det.ctypes.data_as(C.c_void_p)))
        return res, det

    def release(self, job_id: int) -> None:
        check(self._L.ps_server_release(self._h, job_id))
        self._jobs.pop(job_id, None)

    def cancel(self, job_id: int) -> None:
        """Take a job that is still queued out of the queue (an admitted job
        runs to its end: RuntimeError)."""
        check(self._L.ps_server_cancel(self._h, job_id))

    def drain(self, timeout_s: float = -1.0) -> None:
        check(self._L.ps_server_drain(self._h, timeout_s))

    def stats(self) -> dict:
        st = ServerStats()
        check(self._L.ps_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.ps_server_destroy(h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            if not _lib.exiting():
                self.close()
        except Exception:
            pass


# -------------------------------------------------------------- job mixes
PS_NOISE = (1e-4, 1e-3, 5e-3)


def _log_uniform_shots(rng: SplitMix64, lo: int, hi: int) -> int:
    s = math.exp(math.log(lo) + rng.uniform() * (math.log(hi) - math.log(lo)))
    return min(hi, max(lo, int(math.ceil(s / 64.0)) * 64))


def uneven_surface_jobs(count: int = 64, seed: int = 12345, distances: Sequence[int] = tuple(range(3, 22, 2)),
                        shots: Tuple[int, int] = (256, 65536), noise: Sequence[float] = PS_NOISE,
                        job_seed_base: int = 12345) -> List[Job]:
    """Rotated surface-code memory jobs of uneven size: distance uniform over
    `distances` (d rounds), shots log-uniform in `shots` rounded up to a
    multiple of 64, p uniform over `noise`; job j draws from seed
    job_seed_base + j.  Circuits of equal (d, p) are shared."""
    rng = SplitMix64(seed)
    cache = {}
    jobs = []
    for j in range(count):
        d = distances[rng.below(len(distances))]
        s = _log_uniform_shots(rng, *shots)
        p = noise[rng.below(len(noise))]
        if (d, p) not in cache:
            cache[(d, p)] = surface_code_memory(d, d, p=p)
        jobs.append(Job(cache[(d, p)], s, job_seed_base + j, d, p))
    return jobs


def poisson_arrivals(rate_per_s: float, duration_s: float, seed: int = 12345) -> List[float]:
    """Arrival times of a Poisson process (exponential gaps, SplitMix64)."""
    rng = SplitMix64(seed ^ 0x5DEECE66D)
    t, out = 0.0, []
    while True:
        u = rng.uniform()
        t += -math.log(1.0 - u) / rate_per_s
        if t >= duration_s:
            return out
        out.append(t)
