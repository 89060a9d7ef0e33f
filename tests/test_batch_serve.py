"""Batches of uneven jobs in one graph launch (ps_batch_*) and the serving
loop (ps_server_*): each job's measurement records are bit-identical to the
same job run alone on a fresh state, and to the CPU oracle."""
import math

import numpy as np
import pytest


def _bits(words, shots):
    """[nm, w] uint64 record words -> [nm, shots] 0/1 (bit s of word k = shot 64k+s)."""
    b = np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")
    return b[:, :shots].astype(np.int32)


# ------------------------------------------------------------------ CPU
def test_uneven_jobs_follow_the_mix():
    from plaquette_simulator.batch import uneven_surface_jobs, PS_NOISE
    jobs = uneven_surface_jobs(64, seed=12345)
    assert len(jobs) == 64
    assert {j.distance for j in jobs} <= set(range(3, 22, 2))
    assert all(256 <= j.shots <= 65536 and j.shots % 64 == 0 for j in jobs)
    assert {j.p for j in jobs} <= set(PS_NOISE)
    assert [j.seed for j in jobs] == list(range(12345, 12345 + 64))
    assert all(j.num_qubits == 2 * j.distance ** 2 - 1 for j in jobs)
    # seeded: the same mix every time
    again = uneven_surface_jobs(64, seed=12345)
    assert [(j.distance, j.shots, j.p) for j in jobs] == [(j.distance, j.shots, j.p) for j in again]
    # log-uniform shots: about half the jobs below the geometric midpoint 4096
    below = sum(j.shots <= 4096 for j in uneven_surface_jobs(2000, seed=7))
    assert 850 < below < 1150


def test_poisson_arrivals_rate():
    from plaquette_simulator.batch import poisson_arrivals
    t = poisson_arrivals(200.0, 60.0, seed=12345)
    assert all(0 < a < 60.0 for a in t) and t == sorted(t)
    assert abs(len(t) - 12000) < 4 * math.sqrt(12000)
    gaps = np.diff(t)
    assert abs(gaps.mean() - 1 / 200.0) < 0.05 / 200.0 * 4


# ------------------------------------------------------------------ GPU
def _small_jobs():
    from plaquette_simulator.batch import Job
    from plaquette_simulator import circuits as C
    spec = [(3, 320, 0.03, 11), (5, 1000, 5e-3, 12), (3, 64, 1e-3, 13), (7, 700, 1e-3, 14),
            (5, 4096, 1e-2, 15), (3, 2000, 5e-3, 16)]
    return [Job(C.surface_code_memory(d, d, p=p), s, seed, d, p) for d, s, p, seed in spec]


def _alone(ps, job, runs=1):
    from plaquette_simulator.circuit import CompiledCircuit
    st = ps.CliffordState(job.num_qubits, job.shots, job.seed, True)
    cc = CompiledCircuit(job.circuit, st, fused=True, graph=True)
    nm = job.circuit.num_measurements()
    w = ((job.shots + 63) // 64 + 1) & ~1
    out = []
    for _ in range(runs):
        cc.run(reset=True)
        res = np.zeros((nm, w), np.uint64)
        det = np.zeros_like(res)
        cc.copy_records_words(res, det)
        out.append((res, det))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("autotune,graph", [(False, True), (True, True), (False, False)])
def test_batch_jobs_match_alone(ps, autotune, graph):
    from plaquette_simulator.batch import Batch
    jobs = _small_jobs()
    b = Batch(jobs, autotune=autotune, graph=graph)
    assert b.stats["num_jobs"] == len(jobs)
    assert b.stats["shot_gates_per_run"] == sum(j.shot_gates() for j in jobs)
    b.run()
    first = [b.records(j) for j in range(len(jobs))]
    b.run()  # a second run draws fresh outcomes, exactly like a second run alone
    second = [b.records(j) for j in range(len(jobs))]
    for j, job in enumerate(jobs):
        alone = _alone(ps, job, runs=2)
        for k, got in enumerate((first[j], second[j])):
            assert np.array_equal(got[0], alone[k][0]), f"job {j} run {k}: results differ"
            assert np.array_equal(got[1], alone[k][1]), f"job {j} run {k}: determined differ"
        if autotune:
            o = b.job_options(j)
            assert o["seg_words"] in (1, 2, 4, 8, 16) and o["meas_words"] in (0, 1, 2, 4)
    b.close()


def _tableau(L, state, n, shots):
    import ctypes as C
    W = 2 * n + 1
    x = np.empty((shots, W, n), dtype=np.int32)
    z = np.empty_like(x)
    r = np.empty((shots, W), dtype=np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    assert L.ps_device_to_host(state, p(x), p(z), p(r)) == 0
    return x, z, r


@pytest.mark.gpu
def test_batch_table_beside_branch_jobs(ps):
    """Jobs of the shared-x/z plan share one job table (three kernels for
    all of them, knobs tuned on the table); a feed-forward job runs its
    per-shot plan on a branch beside them.  Every job's records and final
    tableau equal the job run alone."""
    from plaquette_simulator import _lib
    from plaquette_simulator.batch import Batch, Job
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    ffc = C.Circuit(4)
    ffc.h(0)
    ffc.m(0)
    ffc.s_if(1, 0)
    ffc.h(1)
    ffc.cx(1, 2)
    ffc.pauli1(3, 0.1, 0.1, 0.1)
    ffc.m(1)
    ffc.m(2)
    ffc.m(3)
    jobs = _small_jobs()[:4] + [Job(ffc, 300, 77, 2, 0.1)]
    b = Batch(jobs, autotune=True, graph=True)
    assert b.stats["table_jobs"] == 4
    assert b.stats["frame_warps"] in (4, 8) and b.stats["bcast_ctas"] in (1, 2)
    b.run()
    L = _lib.load()
    for j, job in enumerate(jobs):
        res, det = b.records(j)
        st = ps.CliffordState(job.num_qubits, job.shots, job.seed, True)
        cc = CompiledCircuit(job.circuit, st, fused=True, graph=True)
        cc.run(reset=True)
        nm = job.circuit.num_measurements()
        w = ((job.shots + 63) // 64 + 1) & ~1
        ares, adet = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
        cc.copy_records_words(ares, adet)
        assert np.array_equal(res, ares) and np.array_equal(det, adet), f"job {j}"
        _, state = b._job(j)
        got = _tableau(L, state, job.num_qubits, job.shots)
        for a, g in zip(st.device_to_host_numpy(), got):
            assert np.array_equal(a, g), f"job {j}: tableau"
    b.close()


@pytest.mark.gpu
def test_batch_job_matches_oracle(ps, O):
    from plaquette_simulator.batch import Batch
    jobs = _small_jobs()[:3]
    b = Batch(jobs, autotune=True)
    b.run()
    for j, job in enumerate(jobs):
        res, det = b.records(j)
        o = O.Oracle(job.num_qubits, job.shots, seed=job.seed)
        o.run(job.circuit.op_array(), job.circuit.param_array())
        gres, gdet = _bits(res, job.shots), _bits(det, job.shots)
        for k in range(job.circuit.num_measurements()):
            ores, odet = o.record(k)
            assert np.array_equal(gres[k], ores), f"job {j} record {k}"
            assert np.array_equal(gdet[k], odet), f"job {j} record {k}"
    b.close()


@pytest.mark.gpu
def test_server_mix_matches_alone(ps):
    from plaquette_simulator.batch import Server
    jobs = _small_jobs() * 2
    biggest = max(j.device_bytes() for j in jobs)
    # A budget of a few jobs: later arrivals queue and are admitted as
    # earlier ones finish, while up to 4 run at once.
    with Server(hbm_budget_bytes=3 * biggest + (64 << 20), max_active=4) as srv:
        ids = [srv.submit(j) for j in jobs]
        got = [srv.records(i) for i in ids]
        infos = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"] <= st["max_latency_s"]
    assert st["pool_peak_bytes"] <= st["pool_bytes"]
    assert all(r["latency_s"] >= 0 and r["admit_s"] >= r["submit_s"] for r in infos)
    for j, job in enumerate(jobs):
        alone = _alone(ps, job)[0]
        assert np.array_equal(got[j][0], alone[0]), f"job {j}: results differ in the mix"
        assert np.array_equal(got[j][1], alone[1]), f"job {j}: determined differ in the mix"


@pytest.mark.gpu
def test_server_refuses_job_over_budget(ps):
    from plaquette_simulator import _lib
    from plaquette_simulator.batch import Server
    job = _small_jobs()[4]
    with Server(hbm_budget_bytes=1 << 20, max_active=2) as srv:
        with pytest.raises(_lib.PlaquetteError) as e:
            srv.submit(job)
        assert e.value.status == _lib.PS_E_NOMEM


@pytest.mark.gpu
def test_server_signs_only_and_feed_forward_jobs(ps):
    """A job with no record-controlled gate holds no per-shot tableaux while
    admitted: its device bytes stay far below its x / z planes alone.  A job
    with one (H on a measured record) keeps them.  Both give the records
    they give alone, in either order of admission."""
    from plaquette_simulator.batch import Job, Server
    from plaquette_simulator import circuits as C
    plain = Job(C.surface_code_memory(9, 3, p=1e-3), 8192, 21, 9, 1e-3)
    ffc = C.Circuit(3)
    ffc.h(0)
    ffc.m(0)
    ffc.h_if(1, 0)
    ffc.cx(1, 2)
    ffc.m(1)
    ffc.m(2)
    ff = Job(ffc, 4096, 22, 3, 0.0)
    for order in ((plain, ff), (ff, plain)):
        with Server(hbm_budget_bytes=1 << 30, max_active=2) as srv:
            ids = [srv.submit(j) for j in order]
            got = [srv.records(i) for i in ids]
            infos = [srv.wait(i) for i in ids]
        for job, (res, det), info in zip(order, got, infos):
            n = job.num_qubits
            w = ((job.shots + 63) // 64 + 1) & ~1
            planes = 2 * (2 * n + 1) * n * w * 8
            if job is plain:
                assert info["device_bytes"] < planes // 4, (info["device_bytes"], planes)
            else:
                assert info["device_bytes"] >= planes
            alone = _alone(ps, job)[0]
            assert np.array_equal(res, alone[0]) and np.array_equal(det, alone[1])


@pytest.mark.gpu
def test_server_park_and_resume(ps):
    """A job served in two parts -- the first kept parked (its tableau and
    event counter in host memory, its device memory freed), the second
    resumed from it -- gives the second part's records, the final tableau
    and event counter exactly as one state running both parts straight
    through.  Feed-forward gates included, so both plans are crossed."""
    from plaquette_simulator.batch import Job, Server
    from plaquette_simulator.circuit import CompiledCircuit
    from drivers import random_mixed_circuit
    n, shots, seed = 10, 64 * 3 + 7, 4242
    a = random_mixed_circuit(n, 250, seed=71)
    b = random_mixed_circuit(n, 250, seed=72)
    with Server(hbm_budget_bytes=1 << 30, max_active=2) as srv:
        i1 = srv.submit(Job(a, shots, seed, 0, 0.0), keep_tableau=True)
        parked = srv.tableau(i1)
        srv.release(i1)
        i2 = srv.submit(Job(b, shots, seed, 0, 0.0), parked=parked, keep_tableau=True)
        res2, det2 = srv.records(i2)
        final = srv.tableau(i2)
        with pytest.raises(Exception):
            srv.tableau(srv.submit(Job(a, shots, seed, 0, 0.0)))  # not kept
    st = ps.CliffordState(n, shots, seed, True)
    CompiledCircuit(a, st, fused=True).run(reset=True)
    assert parked["events"] == st.event_counter()
    cb = CompiledCircuit(b, st, fused=True)
    cb.run(reset=False)
    nm, w = b.num_measurements(), ((shots + 63) // 64 + 1) & ~1
    rres, rdet = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
    cb.copy_records_words(rres, rdet)
    assert np.array_equal(res2, rres) and np.array_equal(det2, rdet)
    x, z, r = st.tableau_words(0, st.words())
    assert np.array_equal(final["x"], x) and np.array_equal(final["z"], z) and np.array_equal(final["r"], r)
    assert final["events"] == st.event_counter()


@pytest.mark.gpu
def test_server_d25_job_matches_oracle(ps, O):
    """The largest serving size (d=25, 1249 qubits): its schedule and tile
    must share one CTA's shared memory; one round, 64 shots, against the
    oracle."""
    from plaquette_simulator.batch import Job, Server
    from plaquette_simulator import circuits as C
    job = Job(C.surface_code_memory(25, 1, p=1e-3), 64, 4321, 25, 1e-3)
    with Server(hbm_budget_bytes=2 << 30, max_active=2) as srv:
        res, det = srv.records(srv.submit(job))
    o = O.Oracle(job.num_qubits, job.shots, seed=job.seed)
    o.run(job.circuit.op_array(), job.circuit.param_array())
    gres, gdet = _bits(res, job.shots), _bits(det, job.shots)
    for k in range(job.circuit.num_measurements()):
        ores, odet = o.record(k)
        assert np.array_equal(gres[k], ores), f"record {k}"
        assert np.array_equal(gdet[k], odet), f"record {k}"


@pytest.mark.gpu
def test_server_failing_job_counted_apart(ps):
    """A job that fails on its worker (its circuit flips on a record that is
    not measured yet: the compile refuses it) is reported failed, not
    completed, leaves no latency behind, and the jobs around it still give
    the records they give alone."""
    from plaquette_simulator import _lib
    from plaquette_simulator.batch import Job, Server
    from plaquette_simulator import circuits as C
    good = _small_jobs()[:3]
    bad_c = C.Circuit(3)
    bad_c.h(0)
    bad_c.h_if(1, 5)
    bad_c.m(0)
    bad = Job(bad_c, 64, 99, 3, 0.0)
    with Server(hbm_budget_bytes=1 << 30, max_active=2) as srv:
        ids = [srv.submit(j) for j in good[:2]] + [srv.submit(bad)] + [srv.submit(good[2])]
        srv.drain(120.0)
        with pytest.raises(_lib.PlaquetteError) as e:
            srv.wait(ids[2], 0.0)
        assert e.value.status == _lib.PS_E_ARG
        got = [srv.records(i) for i in ids[:2] + ids[3:]]
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 3 and st["submitted"] == 4
    for job, (res, det) in zip(good, got):
        alone = _alone(ps, job)[0]
        assert np.array_equal(res, alone[0]) and np.array_equal(det, alone[1])


@pytest.mark.gpu
def test_server_cancel_queued_job(ps):
    """A job cancelled while queued is never admitted and reports
    PS_E_STATE; one already admitted cannot be cancelled and runs to its
    end.  One slot, so the later submissions queue behind the first."""
    from plaquette_simulator import _lib
    from plaquette_simulator.batch import Job, Server
    from plaquette_simulator import circuits as C
    first = Job(C.surface_code_memory(9, 9, p=1e-3), 16384, 7, 9, 1e-3)
    later = _small_jobs()[:3]
    with Server(hbm_budget_bytes=4 << 30, max_active=1) as srv:
        i0 = srv.submit(first)
        ids = [srv.submit(j) for j in later]
        try:
            srv.cancel(ids[2])
            cancelled = True
        except _lib.PlaquetteError as e:  # admitted already: allowed only with the state error
            assert e.status == _lib.PS_E_STATE
            cancelled = False
        with pytest.raises(_lib.PlaquetteError) as e:
            srv.cancel(i0 + 1000)
        assert e.value.status == _lib.PS_E_RANGE
        srv.drain(120.0)
        st = srv.stats()
        if cancelled:
            with pytest.raises(_lib.PlaquetteError) as e:
                srv.wait(ids[2], 0.0)
            assert e.value.status == _lib.PS_E_STATE
            assert st["cancelled"] == 1 and st["completed"] == 3
        else:
            assert st["cancelled"] == 0 and st["completed"] == 4
        assert st["failed"] == 0
