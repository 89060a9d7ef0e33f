"""Shared-x/z runs (fused runs from |0...0> of circuits without per-shot
conditional gates): the x / z bits simulated once on the host, a sign
program per shot-word on the device, the final x / z broadcast to every shot.
Every run here is checked bit for bit against the CPU oracle (whole tableau
and every record) or, where the oracle cannot hold the state, against the
per-shot plan of the same library."""
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


def _random_measure_circuit(n, rounds, seed):
    """Many random-branch measurements and resets: H layers, entangling CX
    chains, biased M and R on every qubit, Pauli gates and channels."""
    from plaquette_simulator import circuits as C
    rng = C.SplitMix64(seed)
    c = C.Circuit(n)
    for _ in range(rounds):
        for q in range(n):
            if rng.below(2):
                c.h(q)
        for q in range(n - 1):
            if rng.below(3) == 0:
                c.cx(q, q + 1)
            if rng.below(5) == 0:
                c.pauli2(q, q + 1, [0.004 * (j + 1) for j in range(15)])
        for q in range(n):
            k = rng.below(6)
            if k == 0:
                c.m(q, bias=0.3)
            elif k == 1:
                c.r(q)
            elif k == 2:
                c.x(q)
            elif k == 3:
                c.pauli1(q, 0.05, 0.02, 0.1)
            else:
                c.m(q)
    return c


def _circuits():
    from plaquette_simulator import circuits as C
    return {
        "mixed_n9": (random_mixed_circuit(9, 400, seed=51, flags=False), 130),
        "mixed_n40": (random_mixed_circuit(40, 700, seed=52, flags=False), 64),
        "mixed_n100": (random_mixed_circuit(100, 900, seed=53, flags=False), 200),
        "random_meas_n30": (_random_measure_circuit(30, 6, seed=54), 192),
        "surface_d3_noisy": (C.surface_code_memory(3, 3, p=0.03), 300),
        "surface_d5_noisy": (C.surface_code_memory(5, 3, p=0.01), 256),
        "clifford_n64": (C.random_clifford(64, 400, seed=55), 128),
    }


@pytest.mark.parametrize("name", list(_circuits().keys()))
@pytest.mark.parametrize("graph", [False, True])
def test_shared_xz_matches_oracle(ps, O, name, graph):
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()[name]
    st = ps.CliffordState(circ.num_qubits, B, 77, True)
    st.apply_hadamard_gate(0)  # the reset must start over from |0...0>
    cc = CompiledCircuit(circ, st, fused=True, graph=graph)
    assert cc.stats["shared_xz"] == 1
    cc.run(reset=True)
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=77)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


@pytest.mark.parametrize("name", ["mixed_n40", "random_meas_n30", "surface_d5_noisy"])
def test_shared_xz_equals_per_shot_plan(ps, name):
    """The same reset run through both plans leaves identical states and records."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()[name]
    out = []
    for shared in (True, False):
        st = ps.CliffordState(circ.num_qubits, B, 9, True)
        cc = CompiledCircuit(circ, st, fused=True, graph=True, shared_xz=shared)
        assert cc.stats["shared_xz"] == (1 if shared else 0)
        cc.run(reset=True)
        st.synchronize()
        recs = [st.record(cc.first_record + k) for k in range(circ.num_measurements())]
        out.append((st.device_to_host_numpy(), recs))
    (a, ra), (b, rb) = out
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    for (u0, u1), (v0, v1) in zip(ra, rb):
        assert np.array_equal(u0, v0) and np.array_equal(u1, v1)


def test_conditional_gates_use_per_shot_plan(ps, O):
    """H_IF / S_IF make the shots' x / z differ: the reset run keeps the
    per-shot plan and still matches the oracle."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ = random_mixed_circuit(12, 400, seed=56, flags=True)
    assert any(op[0] in (11, 12) for op in circ.op_array())
    B = 100
    st = ps.CliffordState(circ.num_qubits, B, 13, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    assert cc.stats["shared_xz"] == 0
    cc.run(reset=True)
    o = O.Oracle(circ.num_qubits, B, seed=13)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


def test_shared_xz_forced_draws(ps, O):
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()["random_meas_n30"]
    nm = circ.num_measurements()
    forced = np.random.default_rng(4).integers(0, 256, size=(nm, (B + 7) // 8), dtype=np.uint8)
    st = ps.CliffordState(circ.num_qubits, B, 6, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.set_forced(forced)
    cc.run(reset=True)
    o = O.Oracle(circ.num_qubits, B, seed=6)
    o.run(circ.op_array(), circ.param_array(), forced)
    _check(st, o, cc.first_record, nm)


def test_shared_xz_then_per_shot_run(ps, O):
    """A reset run (shared x/z) and then a run without reset (per-shot plan
    on the broadcast tableau), and a second reset run: every run draws fresh
    events, exactly like the oracle running the circuit three times."""
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _circuits()["surface_d3_noisy"]
    nm = circ.num_measurements()
    st = ps.CliffordState(circ.num_qubits, B, 15, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    o = O.Oracle(circ.num_qubits, B, seed=15)
    cc.run(reset=True)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, nm)
    cc.run(reset=False)
    o.run(circ.op_array(), circ.param_array())
    st.synchronize()
    for k in range(nm):
        assert np.array_equal(st.record(cc.first_record + k)[0], o.record(nm + k)[0]), f"run 2 record {k}"
    gx, gz, gr = st.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(gx, ox) and np.array_equal(gz, oz) and np.array_equal(gr, orr)
    cc.run(reset=True)
    o.reset()
    o.run(circ.op_array(), circ.param_array())
    st.synchronize()
    for k in range(nm):
        assert np.array_equal(st.record(cc.first_record + k)[0], o.record(2 * nm + k)[0]), f"run 3 record {k}"
    gx, gz, gr = st.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(gx, ox) and np.array_equal(gz, oz) and np.array_equal(gr, orr)


def test_shared_xz_large_register(ps, O):
    """A 40-qubit circuit inside a 3,100-qubit register: the signs of one
    shot-word (6,201 rows) take more than 48 KB of shared memory, and the
    per-shot kernels do not take that many qubits at all.  Qubits 40.. stay
    untouched, so the records equal the 40-qubit oracle's bit for bit and the
    tableau is the oracle's, embedded (rows i, n+i, 2n), around identity."""
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    small = random_mixed_circuit(40, 900, seed=57, flags=False)
    n, m, B = 3100, 40, 128
    big = C.Circuit(n)
    big.ops = list(small.ops)
    big.params = list(small.params)
    st = ps.CliffordState(n, B, 21, True)
    cc = CompiledCircuit(big, st, fused=True, graph=True)
    assert cc.stats["shared_xz"] == 1
    cc.run(reset=True)
    st.synchronize()
    o = O.Oracle(m, B, seed=21)
    o.run(small.op_array(), small.param_array())
    for k in range(small.num_measurements()):
        gres, gdet = st.record(cc.first_record + k)
        ores, odet = o.record(k)
        assert np.array_equal(gres, ores) and np.array_equal(gdet, odet), f"record {k}"
    x, z, r = st.tableau_words(0, 2)  # [2n+1, n, 2] words of the 128 shots
    bits = lambda a: np.unpackbits(np.ascontiguousarray(a).view(np.uint8), axis=-1, bitorder="little")[..., :B]
    ox, oz, orr = o.tableau()  # [B, 2m+1, m]
    rows = list(range(m)) + [n + i for i in range(m)] + [2 * n]
    orows = list(range(m)) + [m + i for i in range(m)] + [2 * m]
    gx = bits(x[rows][:, :m, :])  # [rows, m, B]
    gz = bits(z[rows][:, :m, :])
    gr = bits(r[rows])
    assert np.array_equal(gx, np.transpose(ox[:, orows, :], (1, 2, 0))), "x differs"
    assert np.array_equal(gz, np.transpose(oz[:, orows, :], (1, 2, 0))), "z differs"
    assert np.array_equal(gr, orr[:, orows].T), "r differs"
    # the untouched qubits: identity rows, no support on the small block
    for i in (m, 1000, n - 1):
        assert (x[i, i] == ~np.uint64(0)).all() and (z[n + i, i] == ~np.uint64(0)).all()
        assert not x[i, :m].any() and not z[n + i, :m].any() and not r[i].any() and not r[n + i].any()
    with pytest.raises(Exception):
        cc.run(reset=False)  # the per-shot plan does not take 3,100 qubits


def _edge_circuits():
    from plaquette_simulator import circuits as C
    no_meas = C.Circuit(6)
    for q in range(6):
        no_meas.h(q)
        no_meas.pauli1(q, 0.1, 0.05, 0.2)
    for q in range(5):
        no_meas.cx(q, q + 1)
        no_meas.pauli2(q, q + 1, [0.01 * (j + 1) for j in range(15)])
    one = C.Circuit(1)
    for _ in range(20):
        one.h(0)
        one.pauli1(0, 0.1, 0.1, 0.1)
        one.m(0)
        one.s(0)
        one.r(0)
    return {
        "no_measurements": (no_meas, 130),
        "no_noise": (random_mixed_circuit(8, 300, seed=58, noise=False, flags=False), 70),
        "empty": (C.Circuit(3), 64),
        "one_qubit": (one, 100),
        "one_shot": (random_mixed_circuit(10, 300, seed=59, flags=False), 1),
        "word_and_one": (random_mixed_circuit(10, 300, seed=60, flags=False), 65),
    }


@pytest.mark.parametrize("name", list(_edge_circuits().keys()))
def test_shared_xz_edge_cases(ps, O, name):
    from plaquette_simulator.circuit import CompiledCircuit
    circ, B = _edge_circuits()[name]
    st = ps.CliffordState(circ.num_qubits, B, 31, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    assert cc.stats["shared_xz"] == 1
    cc.run(reset=True)
    st.synchronize()
    o = O.Oracle(circ.num_qubits, B, seed=31)
    o.run(circ.op_array(), circ.param_array())
    _check(st, o, cc.first_record, circ.num_measurements())


def test_compile_cache_reuses_plans(ps, O):
    """A circuit compiled again (another state, other shots, another seed)
    takes its host plan from the compile cache and still matches the oracle
    bit for bit; a changed parameter table is a different key."""
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit, compile_cache_clear, compile_cache_stats
    compile_cache_clear()
    circ = C.surface_code_memory(3, 3, p=0.02)
    for k, (B, seed) in enumerate([(130, 5), (64, 6), (200, 7)]):
        st = ps.CliffordState(circ.num_qubits, B, seed, True)
        cc = CompiledCircuit(circ, st, fused=True, graph=True)
        cc.run(reset=True)
        st.synchronize()
        o = O.Oracle(circ.num_qubits, B, seed=seed)
        o.run(circ.op_array(), circ.param_array())
        gx, gz, gr = st.device_to_host_numpy()
        ox, oz, orr = o.tableau()
        assert np.array_equal(gx, ox) and np.array_equal(gz, oz) and np.array_equal(gr, orr)
        for rid in range(circ.num_measurements()):
            assert np.array_equal(st.record(cc.first_record + rid)[0], o.record(rid)[0])
        stats = compile_cache_stats()
        assert stats["misses"] == 1 and stats["hits"] == k
    other = C.surface_code_memory(3, 3, p=0.03)
    st = ps.CliffordState(other.num_qubits, 64, 1, True)
    CompiledCircuit(other, st, fused=True, graph=True)
    assert compile_cache_stats()["misses"] == 2
