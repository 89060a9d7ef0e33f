"""Circuit format and workload generators (CPU)."""
import os

import numpy as np
import pytest

from plaquette_simulator import circuits as C


def test_parse_reference_format():
    # CliffordCircuit.hpp:32-66: NAME q..., CX/CZ on consecutive pairs;
    # the reference's Execute1 test text (Test_CliffordCircuit.hpp:83).
    c = C.parse_text("H 0\n S 0\n S 0\n H 0\n M 0", 3)
    assert len(c) == 5 and c.num_gates() == 5
    c = C.parse_text("CX 0 1 2 3\nM 0 1 2 3\n", 4)
    assert [o[0] for o in c.ops] == [C.OP_CX, C.OP_CX] + [C.OP_M] * 4
    assert c.ops[1][1:3] == (2, 3)


def test_parse_errors():
    with pytest.raises(ValueError, match="Unsupported operation"):
        C.parse_text("FOO 1\n", 2)
    with pytest.raises(ValueError):
        C.parse_text("M 0 1 2 3\n", 3)  # qubit 3 of 3 (unchecked in the reference)
    with pytest.raises(ValueError):
        C.parse_text("CX 0 1 2\n", 3)


def test_parse_channels_and_roundtrip():
    text = "H 0\nE_PAULI 0.1 0.2 0.3 0 1\nE_PAULI2 " + " ".join(["0.01"] * 15) + " 0 1\nR 1\nMB 0.25 0\n"
    c = C.parse_text(text, 2)
    assert [o[0] for o in c.ops] == [C.OP_H, C.OP_PAULI1, C.OP_PAULI1, C.OP_PAULI2, C.OP_R, C.OP_M]
    c2 = C.parse_text(c.to_text(), 2)
    assert c2.ops == c.ops and np.allclose(c2.params, c.params)


def test_splitmix64_reference_values():
    # SplitMix64 from seed 0: first outputs (Steele, Lea, Flood 2014)
    r = C.SplitMix64(0)
    assert [r.next() for _ in range(3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_random_clifford_shape():
    c = C.random_clifford(64, 1000, seed=12345)
    assert len(c) == 1064 and c.num_gates() == 1064
    ops = c.op_array()
    assert set(ops[:1000, 0].tolist()) <= {C.OP_H, C.OP_S, C.OP_CX}
    cx = ops[ops[:, 0] == C.OP_CX]
    assert (cx[:, 1] != cx[:, 2]).all()


@pytest.mark.parametrize("d", [3, 5, 7, 15])
def test_surface_code_layout(d):
    lay = C.surface_code_layout(d)
    assert len(lay.data) == d * d
    assert len(lay.x_anc) == len(lay.z_anc) == (d * d - 1) // 2
    c = C.surface_code_memory(d, d, p=0.0)
    per_round = 4 * d * (d - 1) + 3 * (d * d - 1)  # CX, H (two layers), M, R
    assert c.num_gates() == d * per_round + d * d
    # every CX layer touches each qubit at most once
    ops = c.op_array()
    cx_rows = np.where(ops[:, 0] == C.OP_CX)[0]
    first_round = cx_rows[: 4 * d * (d - 1)]
    layer = len(first_round) // 4
    for k in range(4):
        qs = ops[first_round[k * layer:(k + 1) * layer]][:, 1:3].reshape(-1)
        assert len(set(qs.tolist())) == len(qs)


def test_surface_code_d15_counts():
    c = C.surface_code_memory(15, 15, p=1e-3)
    assert c.num_qubits == 449
    assert c.num_gates() == 22905  # 15 * 1512 + 225
    assert sum(1 for o in c.ops if o[0] in (C.OP_PAULI1, C.OP_PAULI2)) == 15 * (224 + 840)


def test_noiseless_surface_code_detectors_on_oracle(O):
    """Noiseless memory: every ancilla outcome repeats across rounds and the
    final data parities reproduce the last Z-stabilizer outcomes."""
    d, rounds, B = 3, 3, 64
    c = C.surface_code_memory(d, rounds, p=0.0)
    lay = C.surface_code_layout(d)
    s = O.Oracle(c.num_qubits, B, seed=3)
    s.run(c.op_array(), c.param_array())
    na = d * d - 1
    rec = [s.record(k)[0] for k in range(c.num_measurements())]
    for r in range(1, rounds):
        for a in range(na):
            assert np.array_equal(rec[r * 2 * na + a], rec[(r - 1) * 2 * na + a])
    data = {lay.data[i]: rec[rounds * 2 * na + i] for i in range(d * d)}
    for a, (ax, ay) in enumerate(lay.z_anc):
        par = np.zeros(B, np.int32)
        for dx, dy in ((1, 1), (1, -1), (-1, 1), (-1, -1)):
            if (ax + dx, ay + dy) in data:
                par ^= data[(ax + dx, ay + dy)]
        assert np.array_equal(par, rec[(rounds - 1) * 2 * na + len(lay.x_anc) + a])


def test_reference_benchmark_circuits_oracle_pinned(O, ref_circuits):
    """The oracle against the reference's own outputs on the reference's 59
    benchmark circuits (benchmarks/circuits.tar.gz, committed as op tables
    with the outputs by make_golden.py): every record bit for bit, and the
    final tableau's digest and checksum."""
    import hashlib
    assert len(ref_circuits["cases"]) == 59
    for case in ref_circuits["cases"]:
        B = case["batch"]
        o = O.Oracle(case["num_qubits"], B, seed=case["seed"])
        o.run(np.array(case["ops"], np.int32).reshape(-1, 4), np.array(case["params"], np.float32),
              np.array(case["forced"], np.uint8))
        for rid, (rb, db) in enumerate(case["records"]):
            res, det = o.record(rid)
            assert np.packbits(res.astype(np.uint8), bitorder="little").tolist() == rb, (case["name"], rid)
            assert np.packbits(det.astype(np.uint8), bitorder="little").tolist() == db, (case["name"], rid)
        h = hashlib.sha256()
        for arr in o.tableau():
            h.update(np.ascontiguousarray(arr, dtype=np.int32).tobytes())
        assert h.hexdigest() == case["tableau_sha256"], case["name"]
        assert o.checksum() == case["checksum"], case["name"]
