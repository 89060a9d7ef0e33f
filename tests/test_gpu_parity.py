"""GPU parity: every call goes through the C ABI (libps_gpu.so) and is
compared bit-for-bit with the CPU oracle (oracle/ps_oracle.c, itself pinned to
the reference) on the same seeded inputs and the same random draws."""
import hashlib

import numpy as np
import pytest

from drivers import random_mixed_circuit, run_ops_gpu

pytestmark = pytest.mark.gpu


def _digest(tab):
    h = hashlib.sha256()
    for a in tab:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


def _compare(g, o, nrec):
    gx, gz, gr = g.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(gx, ox), "x differs"
    assert np.array_equal(gz, oz), "z differs"
    assert np.array_equal(gr, orr), "r differs"
    for rid in range(nrec):
        gres, gdet = g.record(rid)
        ores, odet = o.record(rid)
        assert np.array_equal(gres, ores), f"record {rid} results differ"
        assert np.array_equal(gdet, odet), f"record {rid} determined flags differ"


def test_init_tableau(ps, kat):
    st = ps.CliffordState(3, 2, 0, True)
    x, z, r = st.device_to_host_numpy()
    for b in range(2):
        assert (x[b] == np.array(kat["init_n3"]["x"])).all()
        assert (z[b] == np.array(kat["init_n3"]["z"])).all()
        assert r[b].tolist() == [0] * 6 + [1]
    assert st.get_num_qubits() == 3 and st.get_batch_size() == 2 and st.get_seed() == 0


def test_checksum_fixture_and_roundtrip(ps, kat):
    f = kat["checksum_fixture"]
    st = ps.CliffordState.from_host(f["x"], f["z"], f["r"], 5, 1)
    assert st.check_sum() == sum(f["x"]) + sum(f["z"]) + sum(f["r"])
    x, z, r = st.device_to_host()
    assert x == f["x"] and z == f["z"] and r == f["r"]


@pytest.mark.parametrize("which", [0, 1])
def test_measure_random_forced_bias(ps, kat, which):
    bias = kat["measure_random_bias"]["bias"][which]
    st = ps.CliffordState(2, 1, -1, True)
    st.apply_hadamard_gate(1); st.apply_phase_gate(1); st.apply_hadamard_gate(0)
    st.apply_control_not_gate(0, 1)
    st.measure_qubit(1, bias, None)
    assert st.check_sum() == kat["measure_random_bias"]["checksum"][which]


def test_measure_determined_nonvalid_fixture(ps, O, kat):
    """The reference's hand-made 5-qubit fixture is not a valid stabilizer
    tableau; with the stabilizer x bits of q cleared, MeasureQubit takes the
    deterministic branch and must reproduce the reference's per-step sign
    rounding exactly."""
    f = kat["fixture5"]
    n = 5
    for q in range(n):
        x = np.array(f["x"], np.int32).reshape(11, 5)
        x[n:2 * n, q] = 0
        st = ps.CliffordState.from_host(x, f["z"], f["r"], n, 1)
        o = O.Oracle(n, 1, host=(x, np.array(f["z"], np.int32), np.array(f["r"], np.int32)))
        st.measure_qubit(q)
        o.measure(q)
        _compare(st, o, 1)


def test_random_branch_nonvalid_fixture(ps, O, kat):
    f = kat["fixture5"]
    for q in range(5):
        for bit in (0, 1):
            st = ps.CliffordState.from_host(f["x"], f["z"], f["r"], 5, 1)
            o = O.Oracle(5, 1, host=tuple(np.array(f[k], np.int32) for k in ("x", "z", "r")))
            forced = np.array([bit], np.uint8)
            st.measure_qubit(q, 0.5, None, forced=forced)
            o.measure(q, 0.5, -1, forced)
            _compare(st, o, 1)


def test_reference_runs_on_gpu(ps, ref_runs):
    """Outputs recorded from the unmodified reference (make_golden.py)."""
    for case in ref_runs["cases"]:
        B = case["batch"]
        st = ps.CliffordState(case["num_qubits"], B, case["seed"], True)
        ops = np.array(case["ops"], np.int32).reshape(-1, 4)
        forced = np.array(case["forced"], np.uint8)
        run_ops_gpu(st, ops, np.array(case["params"], np.float32), forced)
        for rid, (rb, db) in enumerate(case["records"]):
            res, det = st.record_bits(rid)
            assert res.tolist() == rb, (case["name"], rid)
            assert det.tolist() == db, (case["name"], rid)
        assert _digest(st.device_to_host_numpy()) == case["tableau_sha256"], case["name"]
        assert st.check_sum() == case["checksum"]


@pytest.mark.parametrize("n,B,seed", [(1, 1, 1), (2, 3, 2), (7, 64, 3), (12, 65, 4), (33, 130, 5),
                                      (5, 300, 6), (70, 100, 7)])
@pytest.mark.parametrize("forced", [True, False])
def test_random_circuits(ps, O, n, B, seed, forced):
    circ = random_mixed_circuit(n, 120, seed)
    nm = circ.num_measurements()
    rng = np.random.default_rng(seed)
    fa = rng.integers(0, 256, size=(max(nm, 1), (B + 7) // 8), dtype=np.uint8) if forced else None
    st = ps.CliffordState(n, B, 100 + seed, True)
    o = O.Oracle(n, B, seed=100 + seed)
    run_ops_gpu(st, circ.op_array(), circ.param_array(), fa)
    o.run(circ.op_array(), circ.param_array(), fa)
    _compare(st, o, nm)


def test_wide_state(ps, O):
    """n > 256: several columns per thread in the deterministic branch."""
    from plaquette_simulator import circuits as C
    n, B = 300, 64
    circ = C.random_clifford(n, 900, seed=77, measure_all=False)
    for q in range(0, n, 7):
        circ.m(q)
    circ.r(5)
    for q in range(0, n, 11):
        circ.m(q)
    st = ps.CliffordState(n, B, 9, True)
    o = O.Oracle(n, B, seed=9)
    run_ops_gpu(st, circ.op_array(), circ.param_array())
    o.run(circ.op_array(), circ.param_array())
    _compare(st, o, circ.num_measurements())


def test_surface_code_noisy_parity(ps, O):
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(3, 3, p=0.02)
    B = 200
    st = ps.CliffordState(circ.num_qubits, B, 4242, True)
    o = O.Oracle(circ.num_qubits, B, seed=4242)
    run_ops_gpu(st, circ.op_array(), circ.param_array())
    o.run(circ.op_array(), circ.param_array())
    _compare(st, o, circ.num_measurements())


def test_protocols_gpu(ps):
    def make(n, b):
        return _Adapter(ps.CliffordState(n, b, 5, True))
    from test_oracle_golden import _run_protocols, distillation_batched
    _run_protocols(make)
    distillation_batched(lambda n, b, seed: _Adapter(ps.CliffordState(n, b, seed, True)))


class _Adapter:
    """Oracle-style call names on top of the public Python API."""

    def __init__(self, st):
        self.st = st

    def h_gate(self, q): self.st.apply_hadamard_gate(q)
    def s_gate(self, q): self.st.apply_phase_gate(q)
    def cx(self, c, t): self.st.apply_control_not_gate(c, t)
    def h_flag(self, q, rec): self.st.apply_hadamard_gate_with_apply_flag(q, rec)
    def s_flag(self, q, rec): self.st.apply_phase_gate_with_apply_flag(q, rec)
    def measure(self, q, bias=0.5): return self.st.measure_qubit(q, bias, None)
    def record(self, rid): return self.st.record(rid)

    def get_measurement(self, rid, shot):
        v = self.st.get_measurement(rid, shot)
        return (v is not None,) + tuple(v)


def test_errors_and_ranges(ps):
    st = ps.CliffordState(3, 10, 0, True)
    assert st.get_measurement(0, 0) is None  # no record yet: nullopt
    mid = st.measure_qubit(0)
    assert st.get_measurement(mid, 9) is not None
    assert st.get_measurement(mid, 10) is None
    with pytest.raises(RuntimeError):
        st.measure_qubit(0, 0.5, 7)  # "Measurement id is out of range."
    with pytest.raises(RuntimeError):
        st.apply_hadamard_gate(3)
    with pytest.raises(RuntimeError):
        st.apply_control_not_gate(1, 1)
    assert "CUDA" in st.get_kokkos_backend()


def test_remeasure_into_existing_id_refreshes(ps):
    st = ps.CliffordState(1, 8, 0, True)
    mid = st.measure_qubit(0)
    assert st.get_measurement(mid, 0) == (0, 1)
    st.apply_pauli_x_gate(0)
    st.measure_qubit(0, 0.5, mid)
    assert st.get_measurement(mid, 0) == (1, 1)


def test_copy_and_reset(ps, O):
    st = ps.CliffordState(4, 70, 3, True)
    st.apply_hadamard_gate(0); st.apply_control_not_gate(0, 1); st.apply_phase_gate(2)
    cp = st.copy()
    assert np.array_equal(cp.device_to_host_numpy()[0], st.device_to_host_numpy()[0])
    st.reset_clifford_state()
    fresh = ps.CliffordState(4, 70, 3, True)
    for a, b in zip(st.device_to_host_numpy(), fresh.device_to_host_numpy()):
        assert np.array_equal(a, b)


def test_native_rng_frequencies(ps):
    """Chi-square test of Bernoulli(bias) frequencies of random outcomes."""
    B = 64 * 256
    st = ps.CliffordState(1, B, 99, True)
    st.apply_hadamard_gate(0)
    for bias in (0.5, 0.2):
        mid = st.measure_qubit(0, bias, None)
        res, det = st.record(mid)
        assert (det == 0).all()
        ones = int(res.sum())
        exp1, exp0 = B * bias, B * (1 - bias)
        chi2 = (ones - exp1) ** 2 / exp1 + ((B - ones) - exp0) ** 2 / exp0
        assert chi2 < 10.83  # p = 0.001, one degree of freedom
        st.apply_hadamard_gate(0)  # back to a random state for the next draw
        st.reset_qubit(0)
        st.apply_hadamard_gate(0)
