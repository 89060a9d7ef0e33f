"""Benchmark: shot-gates/s of the rotated surface-code memory circuit at d=15
on one GB300 (fused + CUDA-graph form), beside the plain per-gate form on the
same GPU and the CPU port of the reference's algorithm on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One "step" is one sampling job: the tableau of all shots re-initialised to
|0...0> and the whole circuit executed (22,905 gates per shot for d=15).
Prints ONE JSON line (rank 0).  For N > 1 (torchrun) the job grows with N:
rank r simulates shots [r*S, (r+1)*S) of one N*S-shot job (one seed, draws
keyed by global shot, no collective on the data path) and the slowest rank's
time is reported.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "plaquette-simulator_gb300")
sys.path.insert(0, os.path.join(PKG, "python"))
sys.path.insert(0, PKG)

METRIC = "shot-gates/s at d=15 surface code, batched vs plain on 1 GB300; p50/p99 job latency"

WORKLOADS = {
    # name: (distance, rounds, p, shots)
    "surface_d15": (15, 15, 1e-3, 16384),
    "surface_d5": (5, 5, 1e-3, 4096),
    # small case for profiler captures: 206 MB tableau, still larger than L2
    "surface_d15_s2048": (15, 15, 1e-3, 2048),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="surface_d15")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-shots", type=int, default=0, help="shots of the CPU sample (0 = auto)")
    ap.add_argument("--batch-jobs", type=int, default=64,
                    help="uneven surface-code jobs in the one-launch batch leg (0 = skip)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="seconds of Poisson arrivals in the serving leg (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving leg: arrivals per second")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="serving leg: HBM admission budget")
    ap.add_argument("--serve-drain-s", type=float, default=180.0, help="serving leg: longest wait for the backlog")
    ap.add_argument("--capacity-rate", type=float, default=4000.0,
                    help="capacity leg: arrivals per second (the same job mix, well above the serving rate)")
    ap.add_argument("--capacity-seconds", type=float, default=10.0,
                    help="capacity leg: seconds of arrivals (0 = skip)")
    ap.add_argument("--ff-blocks", type=int, default=90,
                    help="feed-forward leg: distillation blocks side by side (5 qubits each; 0 = skip)")
    return ap.parse_args()


# DRAM bytes (read + written) per shot-word of one x / z broadcast launch of
# the d = 15 circuit, from an ncu capture at 16,384 shots (256 shot-words):
# two launches averaged 0.166 MB read + 1589.37 MB written.
BCAST_DRAM_BYTES_D15_PER_WORD = (0.166e6 + 1589.37e6) / 256


def noisy_ranges(circ) -> int:
    """Runs of non-measurement ops that hold a Pauli channel: the ranges
    the noise kernel writes a vector for."""
    from plaquette_simulator import circuits as C
    n, seen = 0, False
    for code, _a, _b, _c in circ.ops:
        if code in (C.OP_M, C.OP_R):
            n += seen
            seen = False
        elif code in (C.OP_PAULI1, C.OP_PAULI2):
            seen = True
    return n + seen


def workload_circuit(name):
    from plaquette_simulator import circuits as C
    d, rounds, p, shots = WORKLOADS[name]
    return C.surface_code_memory(d, rounds, p=p), shots, {"distance": d, "rounds": rounds, "p": p}


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def host_cpu():
    """The host's core count and CPU model (lscpu), for the CPU baselines."""
    info = {"cores": os.cpu_count() or 1, "model": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                info["model"] = ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


# ------------------------------------------------------------- CPU legs
def cpu_sample(circ, seed: int, shots: int):
    """Time the CPU port of the reference's algorithm (oracle/, int32 tableau,
    flag-gate noise) on `shots` shots.  Returns (seconds, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    threads = os.cpu_count() or 1
    oracle.lib().ora_set_threads(threads)
    o = oracle.Oracle(circ.num_qubits, shots, seed=seed)
    t0 = time.perf_counter()
    o.run(circ.op_array(), circ.param_array())
    return time.perf_counter() - t0, threads


def cpu_baseline(circ, seed, requested_shots=0):
    gates = circ.num_gates()
    shots = requested_shots or 64
    secs, threads = cpu_sample(circ, seed, shots)
    if not requested_shots and secs < 5.0:
        shots = int(min(512, max(64, shots * 10.0 / max(secs, 1e-3))) // 64 * 64) or 64
        secs, threads = cpu_sample(circ, seed, shots)
    return {"value": gates * shots / secs, "unit": "shot-gates/s", "cores": threads, "kind": "port",
            "cpu_model": host_cpu()["model"],
            "sample": f"{shots} shots of the same circuit ({gates} gates/shot) on the C restatement of the "
                      f"reference's algorithm in its int32 layout, OpenMP over {threads} threads: {secs:.2f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    circ, shots, meta = workload_circuit(args.workload)
    gates = circ.num_gates()
    sample = args.cpu_shots or 128
    for _ in range(args.warmup):
        cpu_sample(circ, 12345, min(sample, 64))
    times = []
    threads = 1
    for _ in range(args.steps):
        secs, threads = cpu_sample(circ, 12345, sample)
        times.append(secs)
    sec = sum(times) / len(times)
    value = gates * sample / sec
    # The same circuit without its channels (the same gates: channels are not
    # counted), once: the reference applies every channel outcome as flag
    # gates (H S S H / S S with the shot's flag), so its noisy and noiseless
    # rates differ.
    from plaquette_simulator import circuits as C
    quiet = C.surface_code_memory(meta["distance"], meta["rounds"], p=0.0)
    qsec, _ = cpu_sample(quiet, 12345, sample)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "shot-gates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32 per tableau bit",
        "data": "synthetic: seeded rotated surface-code memory circuit, Philox4x32-10 draws",
        "config": {"workload": f"surface_code_memory d={meta['distance']} rounds={meta['rounds']} "
                               f"p={meta['p']} Z-basis", "num_qubits": circ.num_qubits, "shots": shots,
                   "gates_per_shot": gates, "sample_shots": sample},
        "cpu_baseline": {"value": value, "unit": "shot-gates/s", "cores": threads, "kind": "port",
                         "cpu_model": host_cpu()["model"],
                         "sample": f"{sample} shots per step of the {shots}-shot workload"},
        "e2e": {"value": value, "unit": "shot-gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "noiseless": {"value": quiet.num_gates() * sample / qsec, "unit": "shot-gates/s",
                      "what": f"the same circuit at p=0, {sample} shots, timed once"},
        "note": "the reference's own CPU build needs Kokkos (not available); its headers compiled on the "
                "project's Kokkos-API shim validate this port in the tests, but only the port travels "
                "to the GPU box (no reference checkout there)",
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- batch and serving
def batch_leg(args, rank, torch):
    """64 uneven surface-code jobs (d in 3..21, d rounds, shots log-uniform in
    [256, 65536], p in {1e-4, 1e-3, 5e-3}) in ONE graph launch per run: one
    job table, so the noise vectors, sign programs and x / z broadcasts of
    all jobs are three kernel launches, with the sign-kernel warps and
    broadcast CTAs chosen by timing the table; beside it the same compiled
    jobs run one after another."""
    from plaquette_simulator.batch import Batch, uneven_surface_jobs
    from plaquette_simulator.circuit import CompiledCircuit
    jobs = uneven_surface_jobs(args.batch_jobs, seed=12345 + 7919 * rank)
    t0 = time.perf_counter()
    b = Batch(jobs, autotune=True, graph=True)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream)
    b.run()
    b.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = max(1, min(3, args.steps))
    e0.record(stream)
    for _ in range(k):
        b.run()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / k
    sg = b.stats["shot_gates_per_run"]
    # the same jobs, one after another (each enqueued launch by launch)
    seq = []
    for j in range(len(jobs)):
        c, _ = b._job(j)
        seq.append(CompiledCircuit._borrowed(c.value, jobs[j].circuit, None))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for cc in seq:
        cc.run(reset=True)
        b._L.ps_device_synchronize()
    seq_ms = (time.perf_counter() - t1) * 1e3
    others = sorted({(jobs[j].distance, *b.job_options(j).values()) for j in range(len(jobs))}) \
        if b.stats["table_jobs"] < len(jobs) else []
    out = {"workload": f"{len(jobs)} uneven rotated surface-code memory jobs, d uniform in 3..21 (d rounds), "
                       "shots log-uniform in [256, 65536], p in {1e-4, 1e-3, 5e-3}, one CUDA graph launch "
                       "over one job table",
           "value": sg / (ms / 1e3), "unit": "shot-gates/s", "ms_per_run": ms, "runs": k,
           "shot_gates_per_run": sg, "tableau_gb": b.stats["tableau_bytes"] / 1e9,
           "launches_per_run": b.stats["launches_per_run"], "setup_s": setup_s,
           "compile_ms": b.stats["compile_ms"], "tune_ms": b.stats["tune_ms"],
           "sequential_ms": seq_ms, "speedup_vs_sequential": seq_ms / ms,
           "table": {"jobs": b.stats["table_jobs"], "frame_warps": b.stats["frame_warps"],
                     "bcast_ctas": b.stats["bcast_ctas"]},
           # per-shot tiles only matter for jobs outside the table
           "per_shot_tiles": [{"d": s[0], "seg_rows": s[1], "seg_words": s[2], "seg_threads": s[3],
                               "meas_words": s[4]} for s in others]}
    del seq
    b.close()
    return out


def serving_leg(args, rank, rate=None, seconds=None):
    """Poisson arrivals of sampling jobs (sizes as the batch leg plus d=25),
    admitted by device bytes against an HBM budget; p50/p99 latency."""
    from plaquette_simulator.batch import Server, poisson_arrivals, uneven_surface_jobs
    rate = args.serve_rate if rate is None else rate
    seconds = args.serve_seconds if seconds is None else seconds
    arrivals = poisson_arrivals(rate, seconds, seed=12345 + rank)
    jobs = uneven_surface_jobs(len(arrivals), seed=24680 + rank, distances=tuple(range(3, 22, 2)) + (25,),
                               job_seed_base=100000)
    offered = sum(j.shot_gates() for j in jobs)
    from plaquette_simulator.circuit import compile_cache_stats
    cache0 = compile_cache_stats()
    import queue
    errors = {}
    with Server(hbm_budget_bytes=int(args.serve_budget_gb * 1e9), max_active=16, autotune=False,
                host_pool_bytes=8 << 30) as srv:
        # A client thread takes each job's result as it finishes and releases
        # its host records (as a caller that consumes its results would), so
        # host memory holds only the jobs in flight.
        from plaquette_simulator import _lib
        done_q = queue.Queue()
        stop = threading.Event()

        def consume():
            while not stop.is_set():
                item = done_q.get()
                if item is None:
                    return
                i, j = item
                while not stop.is_set():
                    try:
                        srv.wait(i, 0.5)
                        srv.release(i)
                        break
                    except _lib.PlaquetteError as e:
                        if e.status == _lib.PS_E_TIMEOUT:
                            continue
                        # a failed job: keep one message per kind
                        errors.setdefault(str(e).split("Error in Plaquette:")[-1].strip()[:160], []).append(
                            {"d": j.distance, "shots": j.shots})
                        break

        client = threading.Thread(target=consume, daemon=True)
        client.start()
        t0 = srv.now()
        ids = []
        for t, j in zip(arrivals, jobs):
            dt = t0 + t - srv.now()
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(j))
            done_q.put((ids[-1], j))
        submit_end = srv.now() - t0
        done_q.put(None)
        drained = True
        try:
            srv.drain(args.serve_drain_s)
        except Exception:
            drained = False
        client.join(timeout=30.0 if drained else 0.0)
        stop.set()  # the server closes only after its client is done with it
        client.join()
        st = srv.stats()
    span = max(1e-9, st["last_done_s"] - st["first_submit_s"])
    cache1 = compile_cache_stats()
    hits, misses = cache1["hits"] - cache0["hits"], cache1["misses"] - cache0["misses"]
    return {"workload": f"Poisson arrivals at {rate:g} jobs/s for {seconds:g} s, "
                        "rotated surface-code memory jobs d in {3..21, 25} (d rounds), shots log-uniform in "
                        f"[256, 65536], admission by device bytes against {args.serve_budget_gb:g} GB",
            "jobs": len(ids), "completed": st["completed"], "failed": st["failed"], "drained": drained,
            "tableau_jobs": st["tableau_jobs"],
            "p50_latency_s": st["p50_latency_s"], "p99_latency_s": st["p99_latency_s"],
            "mean_latency_s": st["mean_latency_s"], "max_latency_s": st["max_latency_s"],
            "value": st["shot_gates_completed"] / span, "unit": "shot-gates/s",
            "offered_shot_gates_per_s": offered / seconds,
            "offered_jobs_per_s": len(ids) / seconds,
            "achieved_jobs_per_s": st["completed"] / span, "submit_span_s": submit_end,
            "pool_peak_gb": st["pool_peak_bytes"] / 1e9, "max_active": 16,
            "compile_cache": {"hits": hits, "misses": misses,
                              "hit_rate": hits / max(1, hits + misses)},
            "errors": {k: v[:4] for k, v in errors.items()}}


def _stream_of(st, torch):
    from plaquette_simulator import _lib
    sp = ctypes.c_void_p()
    _lib.check(_lib.load().ps_get_stream(st.handle, ctypes.byref(sp)))
    return torch.cuda.ExternalStream(sp.value)


def feed_forward_leg(args, shots, seed, torch, stream_of):
    """Circuits with per-shot feed-forward (H / S conditioned on each shot's
    own measurement: the reference's ApplyFlag gates) take the per-shot
    plan.  Workload: the batched low-space S-state distillation protocol
    (Test_CliffordState.hpp:675-741), --ff-blocks blocks of 5 qubits side by
    side, every shot of the headline's shot count.  Each step starts from
    |0...0>; the protocol's own check (data qubits 0..2 read 0, qubit 3
    reads 1, all determined, in every shot) is verified on the last step."""
    import numpy as np
    from plaquette_simulator import CliffordState, circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    circ = C.distillation_blocks(args.ff_blocks)
    flag = sum(1 for o in circ.ops if o[0] in (C.OP_H_IF, C.OP_S_IF))
    gates = circ.num_gates() + flag
    st = CliffordState(circ.num_qubits, shots, seed, True)
    stream = stream_of(st, torch)
    out = {"workload": f"S-state distillation, {args.ff_blocks} blocks of 5 qubits ({circ.num_qubits} qubits), "
                       f"{shots} shots, per-shot plan (H_IF / S_IF feed-forward)",
           "num_qubits": circ.num_qubits, "gates_per_shot": gates, "flag_gates_per_shot": flag,
           "measurements": circ.num_measurements(), "unit": "shot-gates/s"}
    for name, fused in (("fused", True), ("plain", False)):
        cc = CompiledCircuit(circ, st, fused=fused, graph=True)
        for _ in range(2 if fused else 1):
            cc.run(reset=True)
        k = max(1, min(args.steps, 5 if fused else 1))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            cc.run(reset=True)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / k
        out[name] = {"ms_per_step": ms, "value": gates * shots / (ms / 1e3), "steps": k,
                     "shared_xz": int(cc.stats["shared_xz"])}
        if fused:
            nm = circ.num_measurements()
            w = ((shots + 63) // 64 + 1) & ~1
            res, det = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
            cc.copy_records_words(res, det)
            b = args.ff_blocks
            tail = slice(nm - 4 * b, nm)
            full = np.uint64(0xFFFFFFFFFFFFFFFF)
            last = shots % 64
            mask = np.full(w, full, np.uint64)
            mask[shots // 64:] = 0
            if last:
                mask[shots // 64] = np.uint64((1 << last) - 1)
            want = np.zeros((4 * b, w), np.uint64)
            want[3 * b:] = mask
            out["protocol_holds"] = bool(np.array_equal(res[tail] & mask, want) and
                                         np.array_equal(det[tail] & mask, np.broadcast_to(mask, det[tail].shape)))
            out["value"] = out["fused"]["value"]
        del cc
    out["speedup_vs_plain"] = out["plain"]["ms_per_step"] / out["fused"]["ms_per_step"]
    del st
    torch.cuda.synchronize()
    return out


def compile_leg(circ, shots, first_shot, seed, gates, world, torch):
    """The host work the timed steps leave out.  compile_ms: ps_circuit_compile
    of the workload on a fresh state, with the compile cache cleared (cold)
    and again (cached).  cold_e2e: one whole sampling job from nothing -- a
    fresh state, the cold compile (graph capture included), one run, every
    record copied to host memory, everything freed -- as shot-gates/s over
    its wall time; cached_e2e: the same with the compile cache warm."""
    import numpy as np
    from plaquette_simulator import CliffordState
    from plaquette_simulator.circuit import CompiledCircuit, compile_cache_clear

    def one_job(clear):
        if clear:
            compile_cache_clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = CliffordState(circ.num_qubits, shots, seed + 1, True)
        st.set_shot_offset(first_shot)
        t1 = time.perf_counter()
        cc = CompiledCircuit(circ, st, fused=True, graph=True)
        t2 = time.perf_counter()
        cc.run(reset=True)
        nm = int(cc.stats["num_measurements"])
        w_words = (((shots + 63) // 64) + 1) & ~1
        res = np.empty((nm, w_words), np.uint64)
        det = np.empty_like(res)
        cc.copy_records_words(res, det)
        del cc, st
        t3 = time.perf_counter()
        return (t2 - t1) * 1e3, (t3 - t0)

    cold_ms, cold_s = one_job(True)
    cached_ms, cached_s = one_job(False)
    return {"compile_ms_cold": cold_ms, "compile_ms_cached": cached_ms,
            "cold_e2e": {"value": gates * shots * world / cold_s, "unit": "shot-gates/s", "seconds": cold_s,
                         "what": "fresh state + cold compile (cache cleared, graph capture) + one run + all "
                                 "records to host + free"},
            "cached_e2e": {"value": gates * shots * world / cached_s, "unit": "shot-gates/s", "seconds": cached_s,
                           "what": "the same with the compile cache warm (a job of a circuit seen before)"},
            "note": "the headline value and e2e time repeated runs of one compiled circuit: compile is outside "
                    "their timed region and reported here"}


# ---------------------------------------------------------------- ours
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import build as psbuild
    psbuild.build()
    from plaquette_simulator import CliffordState, _lib
    from plaquette_simulator.circuit import CompiledCircuit

    L = _lib.load()
    _lib.check(L.ps_set_device(local))
    circ, shots, meta = workload_circuit(args.workload)
    gates = circ.num_gates()
    # Weak scaling over one job: rank r holds shots [r*S, (r+1)*S) of a
    # world*S-shot job with one seed (draws keyed by global shot).
    from plaquette_simulator.shard import weak_range
    seed = 12345
    first_shot, _ = weak_range(shots, rank)
    st = CliffordState(circ.num_qubits, shots, seed, True)
    st.set_shot_offset(first_shot)
    fused = CompiledCircuit(circ, st, fused=True, graph=True)
    sp = ctypes.c_void_p()
    _lib.check(L.ps_get_stream(st.handle, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def time_steps(cc, k):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(k):
            cc.run(reset=True)
        e1.record(stream)
        e1.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / k
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    for _ in range(max(3, args.warmup)):
        fused.run(reset=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_steps(fused, args.steps)
    value = gates * shots * world / (ms / 1e3)
    clocks = clk.summary()

    # ---- e2e: the same job through the C ABI with the records read back to
    # pinned host memory every step.
    nm = int(fused.stats["num_measurements"])
    w_words = (((shots + 63) // 64) + 1) & ~1
    res_h = torch.empty((nm, w_words), dtype=torch.int64, pin_memory=True)
    det_h = torch.empty_like(res_h, pin_memory=True)
    barrier()
    t0 = time.perf_counter()
    wds = 0
    for _ in range(args.steps):
        fused.run(reset=True)
        wds = fused.copy_records_words(res_h.numpy(), det_h.numpy())
    barrier()
    e2e_sync_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    # Pipelined: two compiled copies of the circuit on the state, run in
    # turn; each run's records go to their own pinned buffers on a copy
    # stream while the next run computes (ps_circuit_copy_records_async).
    # Every step still copies its run parameters in and all its records out.
    twin = CompiledCircuit(circ, st, fused=True, graph=True, shared_xz=bool(fused.stats["shared_xz"]))
    pair = [fused, twin]
    bufs = [(res_h, det_h), (torch.empty_like(res_h, pin_memory=True), torch.empty_like(det_h, pin_memory=True))]
    for cc in pair:  # warm the twin
        cc.run(reset=True)
        cc.copy_records_words(bufs[0][0].numpy(), bufs[0][1].numpy())
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        cc = pair[k % 2]
        if k >= 2:
            cc.wait_records()  # its buffers are free again
        cc.run(reset=True)
        cc.copy_records_async(bufs[k % 2][0].numpy(), bufs[k % 2][1].numpy())
    for cc in pair:
        cc.wait_records()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    del twin
    if dist:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    d2h = 2 * nm * wds * 8

    # ---- roofline: per-kind device time of one run (events around launches)
    prof = fused.profile(reset=True)
    shared = bool(fused.stats["shared_xz"])
    n_q = circ.num_qubits
    W = 2 * n_q + 1
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    seg_bytes = meas_bytes = None
    if shared:
        # Algorithmic bytes of the shared-x/z plan (per run):
        #  sign program (one launch): the final signs of every row and
        #    shot-word written once, plus the records (result + determined
        #    words per measurement);
        #  x / z broadcast: the x and z words of every row, qubit and
        #    shot-word written once.
        #  channel noise: the XOR vector of every range with channels and
        #    every shot-word written once (W rounded up to even words).
        kind_bytes = {
            "sign_program": W * w_words * 8 + 2 * nm * w_words * 8,
            "xz_broadcast": 2 * W * n_q * w_words * 8,
            "channel_sample": noisy_ranges(circ) * w_words * (W + 1) // 2 * 2 * 8,
        }
        kernel_of = {"sign_program": "frame_run_kernel", "xz_broadcast": "broadcast_jobs_kernel",
                     "channel_sample": "noise_vec_kernel"}
    else:
        meas_bytes = fused.measure_bytes(reset=True)
        seg_bytes = float(fused.stats["segment_bytes"])
        kind_bytes = {"segment": seg_bytes, "measure": meas_bytes}
        kernel_of = {"segment": "segment_kernel", "measure": "measure_kernel"}
    dom = max(kind_bytes, key=lambda k: prof[k]["ms"])
    dom_bytes, dom_ms = kind_bytes[dom], prof[dom]["ms"]
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    traffic = None
    if dom == "segment" and meta["distance"] == 15:
        # DRAM bytes per segment launch from one ncu capture of the d=15
        # circuit at 32 shot-words (207.1 MB read + 147.9 MB written),
        # scaled by shot-words.
        traffic = (207.1e6 + 147.9e6) / 32 * w_words
    elif dom == "xz_broadcast" and meta["distance"] == 15 and BCAST_DRAM_BYTES_D15_PER_WORD:
        # DRAM bytes of one broadcast launch from an ncu capture of the d=15
        # workload at 16,384 shots (dram__bytes_read.sum +
        # dram__bytes_write.sum), per shot-word.
        traffic = BCAST_DRAM_BYTES_D15_PER_WORD * w_words
    roofline = {"bound": "hbm", "kernel": kernel_of[dom],
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s",
                "traffic": traffic,
                "algorithmic_bytes_per_launch": dom_bytes / max(1, prof[dom]["launches"]),
                "avg_launch_ms": dom_ms / max(1, prof[dom]["launches"]),
                "kinds": {k: {"ms": round(prof[k]["ms"], 4), "launches": prof[k]["launches"],
                              "algorithmic_GBps": kind_bytes[k] / max(1e-9, prof[k]["ms"] / 1e3) / 1e9}
                          for k in kind_bytes}}
    if dom == "sign_program":
        roofline["note"] = ("latency-bound: one CTA per shot-word runs the whole sign program on signs held in "
                            "shared memory; it moves little HBM data by design")
    elif dom == "xz_broadcast":
        roofline["note"] = ("the broadcast writes the final x / z bits of every row, qubit and shot; in the run "
                            "it overlaps the sign kernel on a side stream (times here are serialised launches)")

    line = {
        "metric": METRIC, "value": value, "unit": "shot-gates/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 bit-packed GF(2) (1 bit per tableau entry)",
        "data": "synthetic: seeded rotated surface-code memory circuit, Philox4x32-10 noise and outcomes",
        "config": {"workload": f"surface_code_memory d={meta['distance']} rounds={meta['rounds']} p={meta['p']} "
                               f"Z-basis, fused + CUDA graph" + (", shared x/z" if shared else ""),
                   "num_qubits": circ.num_qubits, "shots": shots, "gates_per_shot": gates,
                   "tableau_bytes": 3 * (2 * circ.num_qubits + 1) * circ.num_qubits * ((shots + 63) // 64) * 8,
                   "l2": "no flush needed: the 2.48 GB tableau (1.65 GB of it the x/z rewritten every step) is larger than the 129 MB L2",
                   "parallelism": f"shots split over {world} GPU(s), {shots} per GPU",
                   "steps": "repeated sampling runs (fresh draws, full tableau and records written) of one "
                            "compiled circuit; compile time and a cold job are reported under compile"},
        # the per-shot plan's reset adds init_zero_kernel; shared-x/z runs start from zero signs in the sign kernel
        "gpu_launches": int(fused.stats["launches_per_run"]) + (0 if shared else 1),
        "clocks": clocks,
        "e2e": {"value": gates * shots * world / (e2e_ms / 1e3), "unit": "shot-gates/s",
                "h2d_bytes_per_step": 16, "d2h_bytes_per_step": d2h,
                "what": "ps_circuit_run + ps_circuit_copy_records_async of every step's records into pinned host "
                        "memory, two compiled copies of the circuit run in turn so that one step's records "
                        "travel while the next step computes (all copies waited for inside the timed region); "
                        "the 16 H2D bytes are the run parameters (seed, event base)",
                "sync": {"value": gates * shots * world / (e2e_sync_ms / 1e3), "ms_per_step": e2e_sync_ms,
                         "what": "one circuit, ps_circuit_run then a blocking ps_circuit_copy_records per step"}},
        "roofline": roofline,
        "profile_ms": {k: round(v["ms"], 3) for k, v in prof.items() if v["launches"]},
        "plan": "shared x/z: x and z simulated once on the host, a sign program per shot-word on the device, "
                "final x / z written to every shot" if shared else "per-shot tableau",
        "algorithmic_bytes_per_step": {k: float(v) for k, v in kind_bytes.items()},
    }

    line["compile"] = compile_leg(circ, shots, first_shot, seed, gates, world, torch)
    if not args.no_plain and shared:
        per_shot = CompiledCircuit(circ, st, fused=True, graph=True, shared_xz=False)
        per_shot.run(reset=True)
        k = max(1, min(3, args.steps))
        qms = time_steps(per_shot, k)
        qprof = per_shot.profile(reset=True)
        line["per_shot_plan"] = {"ms_per_step": qms, "value": gates * shots * world / (qms / 1e3), "steps": k,
                                 "profile_ms": {kk: round(v["ms"], 3) for kk, v in qprof.items() if v["launches"]},
                                 "form": "fused segments and measurement phases over every shot's tableau"}
        del per_shot
    if not args.no_plain:
        plain = CompiledCircuit(circ, st, fused=False, graph=True)
        plain.run(reset=True)
        k = max(1, min(2, args.steps))
        pms = time_steps(plain, k)
        line["plain"] = {"ms_per_step": pms, "value": gates * shots * world / (pms / 1e3), "steps": k,
                         "launches_per_step": int(plain.stats["launches_per_run"]) + 1,
                         "form": "one kernel launch per op, captured in a CUDA graph"}
        line["speedup_vs_plain"] = pms / ms
        del plain

    del fused, st
    torch.cuda.synchronize()
    if args.ff_blocks > 0 and world == 1:
        line["feed_forward"] = feed_forward_leg(args, shots, seed, torch, stream_of=_stream_of)
    if args.batch_jobs > 0:
        line["batch"] = batch_leg(args, rank, torch)
    if args.serve_seconds > 0:
        line["serving"] = serving_leg(args, rank)
        line["p50_latency_s"] = line["serving"]["p50_latency_s"]
        line["p99_latency_s"] = line["serving"]["p99_latency_s"]
    if args.capacity_seconds > 0:
        # the same job mix offered far above the serving rate: what the
        # server completes per second once it is the bottleneck
        line["serving_capacity"] = serving_leg(args, rank, args.capacity_rate, args.capacity_seconds)

    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(circ, seed, args.cpu_shots)

    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
