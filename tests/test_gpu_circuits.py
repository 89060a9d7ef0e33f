"""Compiled circuits (plain and fused forms, with and without CUDA graphs)
against the CPU oracle, bit-for-bit, through the C ABI."""
import numpy as np
import pytest

from drivers import random_mixed_circuit

pytestmark = pytest.mark.gpu


def _check(st, o, first, nm):
    gx, gz, gr = st.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(gx, ox), "x differs"
    assert np.array_equal(gz, oz), "z differs"
    assert np.array_equal(gr, orr), "r differs"
    for k in range(nm):
        gres, gdet = st.record(first + k)
        ores, odet = o.record(k)
        assert np.array_equal(gres, ores), f"record {k} results differ"
        assert np.array_equal(gdet, odet), f"record {k} determined differ"


def _circuits():
    from plaquette_simulator import circuits as C
    return {
        "mixed_n9": (random_mixed_circuit(9, 300, seed=31), 130),
        "mixed_n40": (random_mixed_circuit(40, 500, seed=32), 64),
        "surface_d3_noisy": (C.surface_code_memory(3, 3, p=0.03), 300),
        "surface_d5_noisy": (C.surface_code_memory(5, 2, p=0.01), 256),
        "clifford_n64": (C.random_clifford(64, 400, seed=33), 128),
    }


@pytest.mark.parametrize("name", list(_circuits().keys()))
@pytest.mark.parametrize("fused,graph", [(False, False), (False, True), (True, False), (True, True)])
def test_compiled_matches_oracle(ps, O, name, fused, graph):
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()[name]
    st = ps.CliffordState(circ.num_qubits, B, 77, True)
    cc = CompiledCircuit(circ, st, fused=fused, graph=graph)
    cc.run()
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=77)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.parametrize("fused", [False, True])
def test_forced_draws(ps, O, fused):
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()["mixed_n40"]
    nm = circ.num_measurements()
    forced = np.random.default_rng(3).integers(0, 256, size=(nm, (B + 7) // 8), dtype=np.uint8)
    st = ps.CliffordState(circ.num_qubits, B, 5, True)
    cc = CompiledCircuit(circ, st, fused=fused, graph=True)
    cc.set_forced(forced)
    cc.run()
    o = O.Oracle(circ.num_qubits, B, seed=5)
    o.run(circ.op_array(), circ.param_array(), forced)
    _check(st, o, cc.first_record, nm)


def test_two_runs_advance_events(ps, O):
    """A second run of the same compiled graph draws fresh events."""
    from plaquette_simulator.circuit import CompiledCircuit
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(3, 2, p=0.05)
    B = 128
    st = ps.CliffordState(circ.num_qubits, B, 11, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.run()
    cc.run()
    o = O.Oracle(circ.num_qubits, B, seed=11)
    o.run(circ.op_array(), circ.param_array())
    o.run(circ.op_array(), circ.param_array())
    # the records hold the second run; the oracle's second run wrote k + nm
    nm = circ.num_measurements()
    st.synchronize()
    for k in range(nm):
        assert np.array_equal(st.record(cc.first_record + k)[0], o.record(nm + k)[0])
    gx, gz, gr = st.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(gr, orr) and np.array_equal(gx, ox)


def test_reset_run_repeats(ps, O):
    from plaquette_simulator.circuit import CompiledCircuit
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(3, 2, p=0.05)
    B = 64
    st = ps.CliffordState(circ.num_qubits, B, 12, True)
    st.apply_hadamard_gate(0)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.run(reset=True)
    o = O.Oracle(circ.num_qubits, B, seed=12)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.parametrize("rows,words,threads", [(1, 2, 64), (1, 4, 128), (2, 4, 256), (1, 16, 256), (2, 8, 256), (4, 2, 128)])
def test_tile_shapes(ps, O, rows, words, threads):
    from plaquette_simulator.circuit import CompiledCircuit
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(5, 2, p=0.02)
    B = 64 * 20 + 7
    st = ps.CliffordState(circ.num_qubits, B, 21, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=False, seg_rows=rows, seg_words=words, seg_threads=threads)
    cc.run()
    o = O.Oracle(circ.num_qubits, B, seed=21)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


def test_fused_on_host_loaded_tableau(ps, O):
    """A tableau loaded from the host is not assumed valid: resets keep their
    X inside the measurement phase, and results stay exact."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ = random_mixed_circuit(6, 200, seed=41)
    B = 70
    rng = np.random.default_rng(9)
    W = 13
    x = rng.integers(0, 2, size=(B, W, 6), dtype=np.int32)
    z = rng.integers(0, 2, size=(B, W, 6), dtype=np.int32)
    r = rng.integers(0, 2, size=(B, W), dtype=np.int32)
    st = ps.CliffordState.from_host(x, z, r, 6, B, 3)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.run()
    o = O.Oracle(6, B, seed=3, host=(x, z, r))
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.gpu
@pytest.mark.parametrize("meas_words", [1, 2, 4])
def test_d15_two_rounds_match_oracle(ps, O, meas_words):
    """449 qubits: measurement windows of up to 16 ancilla measure+resets at
    the end (no later segment to defer the resets into), shared-memory sizes
    between the small and the large configurations."""
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    circ = C.surface_code_memory(15, 2, p=2e-3)
    B = 256
    st = ps.CliffordState(circ.num_qubits, B, 99, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True, meas_words=meas_words)
    cc.run()
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=99)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["surface_d3_noisy", "surface_d5_noisy", "mixed_n40"])
@pytest.mark.parametrize("form,words", [("warp", 8), ("resident", 8), ("word", 1), ("word", 2), ("word", 4),
                                        ("word", 8), ("word", 16)])
def test_segment_forms_match_oracle(ps, O, name, form, words):
    """Every fused-segment form: one warp per (row, word) with every gate
    through shared memory; the register-resident form (gate-dense columns in
    registers, channel outcomes and sign ops through their propagated
    Paulis); the word-vector form (one thread per gate over all words of a
    one-row tile)."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()[name]
    B = max(B, 64 * words + 5)
    st = ps.CliffordState(circ.num_qubits, B, 123, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True, resident=form == "resident",
                         word_vector=form == "word", seg_rows=1, seg_words=words,
                         seg_threads=256 if words >= 4 else 64)
    if form == "resident" and name.startswith("surface"):
        assert cc.stats["resident_segments"] == cc.stats["num_segments"] > 0
    if form != "resident":
        assert cc.stats["resident_segments"] == 0
    cc.run()
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=123)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mixed_n9", "mixed_n40", "clifford_n64", "surface_d5_noisy"])
@pytest.mark.parametrize("meas_words", [1, 2, 4])
def test_words_per_cta_match_oracle(ps, O, name, meas_words):
    """The measurement kernel with 1, 2 and 4 shot-words per CTA (random
    branches with per-shot pivots, uniform pivots, deterministic windows)."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ, _ = _circuits()[name]
    B = 256 + 64 * 3  # 7 words (odd: padded to 8)
    st = ps.CliffordState(circ.num_qubits, B, 31, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True, meas_words=meas_words)
    cc.run()
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=31)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.parametrize("form", ["per_op", "plain", "fused", "fused_graph"])
def test_reference_benchmark_circuits_on_gpu(ps, ref_circuits, form):
    """The reference's 59 benchmark circuits (benchmarks/circuits.tar.gz, in
    the line format of CliffordCircuit.hpp:32-66) against the reference's own
    outputs (tests/golden/reference_circuits.json): op by op through the C
    ABI, and compiled in the plain and fused forms; every record and the
    final tableau, bit for bit."""
    import hashlib
    from drivers import run_ops_gpu
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    for case in ref_circuits["cases"]:
        B = case["batch"]
        ops = np.array(case["ops"], np.int32).reshape(-1, 4)
        params = np.array(case["params"], np.float32)
        forced = np.array(case["forced"], np.uint8)
        st = ps.CliffordState(case["num_qubits"], B, case["seed"], True)
        first = 0
        if form == "per_op":
            run_ops_gpu(st, ops, params, forced)
        else:
            circ = C.Circuit(case["num_qubits"])
            circ.ops = [tuple(int(v) for v in row) for row in ops]
            circ.params = [float(v) for v in params]
            cc = CompiledCircuit(circ, st, fused=form != "plain", graph=form == "fused_graph")
            if case["records"]:
                cc.set_forced(forced)
            cc.run(reset=False)
            first = cc.first_record
        for rid, (rb, db) in enumerate(case["records"]):
            res, det = st.record_bits(first + rid)
            assert res.tolist() == rb, (form, case["name"], rid)
            assert det.tolist() == db, (form, case["name"], rid)
        h = hashlib.sha256()
        for arr in st.device_to_host_numpy():
            h.update(np.ascontiguousarray(arr, dtype=np.int32).tobytes())
        assert h.hexdigest() == case["tableau_sha256"], (form, case["name"])
        assert st.check_sum() == case["checksum"], (form, case["name"])


_CONFIG_ORACLE = {}


def _config(name):
    """The two CPU-sized workloads of the benchmark definition at their full
    sizes: n = 64 random {H, S, CX} circuit of 1000 gates then M on every
    qubit, 1024 shots; the d = 5 rotated surface-code memory, 5 rounds,
    p = 1e-3, 4096 shots.  Seed 12345, native (Philox) draws."""
    from plaquette_simulator import circuits as C
    if name == "clifford_n64_1000g_s1024":
        return C.random_clifford(64, 1000, seed=12345), 1024
    return C.surface_code_memory(5, 5, p=1e-3), 4096


@pytest.mark.parametrize("name", ["clifford_n64_1000g_s1024", "surface_d5_r5_p1e-3_s4096"])
@pytest.mark.parametrize("form", ["plain", "fused_per_shot", "fused_shared_xz"])
def test_baseline_configs_full_size(ps, O, name, form):
    """Whole tableau and every record of each shot against the oracle (run
    once per workload), bit for bit."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _config(name)
    if name not in _CONFIG_ORACLE:
        o = O.Oracle(circ.num_qubits, B, seed=12345)
        o.run(circ.op_array(), circ.param_array())
        _CONFIG_ORACLE[name] = o
    o = _CONFIG_ORACLE[name]
    st = ps.CliffordState(circ.num_qubits, B, 12345, True)
    cc = CompiledCircuit(circ, st, fused=form != "plain", graph=True, shared_xz=form == "fused_shared_xz")
    assert bool(cc.stats["shared_xz"]) == (form == "fused_shared_xz")
    cc.run(reset=True)
    st.synchronize()
    _check(st, o, cc.first_record, circ.num_measurements())
