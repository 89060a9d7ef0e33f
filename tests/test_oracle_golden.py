"""Pins the CPU oracle (oracle/ps_oracle.c) to the reference's own golden
vectors (plaquette_simulator/src/tests/Test_CliffordState.hpp, read into
tests/golden/reference_kat.json) and to recorded outputs of the reference
itself (tests/golden/reference_runs.json)."""
import hashlib

import numpy as np
import pytest


def _fixture(kat, key="fixture5"):
    f = kat[key]
    return f["n"], np.array(f["x"], np.int32), np.array(f["z"], np.int32), np.array(f["r"], np.int32)


def test_init_tableau(O, kat):
    # Test_CliffordState.hpp:29-64
    s = O.Oracle(3, 2)
    x, z, r = s.tableau()
    for b in range(2):
        assert (x[b] == np.array(kat["init_n3"]["x"])).all()
        assert (z[b] == np.array(kat["init_n3"]["z"])).all()
        assert r[b].tolist() == [0] * 6 + [1]


def test_pauli_product_phase_table(O, kat):
    # Test_CliffordState.hpp:160-174
    L = O.lib()
    P, E = kat["pauli_product_phase"]["paulis"], kat["pauli_product_phase"]["expected"]
    assert L.ora_pauli_product_phase(1, 0, 1, 1) == 1
    for i in range(4):
        for j in range(4):
            assert L.ora_pauli_product_phase(P[i][0], P[i][1], P[j][0], P[j][1]) == E[i][j]


def test_checksum_fixture(O, kat):
    # Test_CliffordState.hpp:176-202
    n, x, z, r = _fixture(kat, "checksum_fixture")
    s = O.Oracle(n, 1, host=(x, z, r))
    assert s.checksum() == int(x.sum() + z.sum() + r.sum())


def test_row_product_sign_golden(O, kat):
    # Test_CliffordState.hpp:204-342: 110 (i, k) pairs on a fresh fixture each
    n, x, z, r = _fixture(kat)
    base = int(x.sum() + z.sum() + r.sum())
    got = 0
    for i, k, want in kat["row_product_sign"]["expected"]:
        s = O.Oracle(n, 1, host=(x, z, r))
        assert s.row_product_sign(0, i, k) == want, (i, k)
        assert s.checksum() == base
        got += 1
    assert got == 110


def test_row_multiply_golden(O, kat):
    # Test_CliffordState.hpp:344-454
    n, x, z, r = _fixture(kat)
    for i, k, want in kat["row_multiply_checksum"]["expected"]:
        s = O.Oracle(n, 1, host=(x, z, r))
        s.row_multiply(0, i, k)
        assert s.checksum() == want, (i, k)


def test_measure_determined_golden(O, kat):
    # Test_CliffordState.hpp:456-511
    n, x, z, r = _fixture(kat)
    for q, want in enumerate(kat["measure_determined"]["expected"]):
        s = O.Oracle(n, 1, host=(x, z, r))
        assert s.measure_determined(0, q) == want


@pytest.mark.parametrize("which", [0, 1])
def test_measure_random_forced_bias(O, kat, which):
    # Test_CliffordState.hpp:513-542: bias 0 / 1 force the random outcome
    bias = kat["measure_random_bias"]["bias"][which]
    want = kat["measure_random_bias"]["checksum"][which]
    s = O.Oracle(2, 1)
    s.h_gate(1); s.s_gate(1); s.h_gate(0); s.cx(0, 1)
    s.measure(1, bias)
    assert s.checksum() == want


def _run_protocols(make):
    """The reference's protocol tests (Test_CliffordState.hpp:66-158,
    :544-741); every assertion holds for any random branch."""
    s = make(1, 1)  # Measure0: HSSH -> |1>
    s.h_gate(0); s.s_gate(0); s.s_gate(0); s.h_gate(0)
    s.measure(0)
    assert s.get_measurement(0, 0)[1:] == (1, 1)
    s = make(1, 1)
    s.measure(0)
    assert s.get_measurement(0, 0)[1] == 0
    s = make(2, 1)  # Measure3
    s.h_gate(0); s.s_gate(0); s.s_gate(0); s.h_gate(0)
    s.measure(0); s.measure(1)
    assert s.get_measurement(0, 0)[1:] == (1, 1)
    assert s.get_measurement(1, 0)[1:] == (0, 1)
    s = make(2, 1)  # EPR
    s.h_gate(0); s.cx(0, 1); s.measure(0); s.measure(1)
    r0, r1 = s.get_measurement(0, 0), s.get_measurement(1, 0)
    assert r0[2] == 0 and r1[2] == 1 and r0[1] == r1[1]


def test_protocols_oracle(O):
    _run_protocols(lambda n, b: O.Oracle(n, b, seed=5))


def test_distillation_batched_oracle(O):
    # Test_CliffordState.hpp:674-741 with flag gates, batch 100
    distillation_batched(lambda n, b, seed: O.Oracle(n, b, seed=seed))


def distillation_batched(make, batch=100, seed=1231232132):
    s = make(5, batch, seed)
    phasors = [[0], [1], [2], [0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]
    anc = 4
    for ph in phasors:
        s.h_gate(anc)
        for k in ph:
            s.cx(anc, k)
        s.h_gate(anc); s.s_gate(anc); s.h_gate(anc)
        mid = s.measure(anc)
        res, det = s.record(mid)
        assert (det == 0).all()
        for k in ph + [anc]:
            s.h_flag(k, mid); s.s_flag(k, mid); s.s_flag(k, mid); s.h_flag(k, mid)
    for k in range(3):
        mid = s.measure(k)
        res, det = s.record(mid)
        assert (res == 0).all() and (det == 1).all()
    s.s_gate(3); s.h_gate(3)
    mid = s.measure(3)
    res, det = s.record(mid)
    assert (res == 1).all() and (det == 1).all()


def test_distillation_seeds_oracle(O):
    # Test_CliffordState.hpp:574-633, 100 seeds, batch 1, host feed-forward
    for seed in range(100):
        s = O.Oracle(5, 1, seed=seed)
        anc = 4
        for ph in [[0], [1], [2], [0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]:
            s.h_gate(anc)
            for k in ph:
                s.cx(anc, k)
            s.h_gate(anc); s.s_gate(anc); s.h_gate(anc)
            mid = s.measure(anc)
            ok, v, d = s.get_measurement(mid, 0)
            assert d == 0
            if v:
                for k in ph + [anc]:
                    s.h_gate(k); s.s_gate(k); s.s_gate(k); s.h_gate(k)
        for k in range(3):
            mid = s.measure(k)
            assert s.get_measurement(mid, 0)[1:] == (0, 1)
        s.s_gate(3); s.h_gate(3)
        mid = s.measure(3)
        assert s.get_measurement(mid, 0)[1:] == (1, 1)


def test_reference_runs_replayed_by_oracle(O, ref_runs):
    """Outputs of the unmodified reference (recorded by make_golden.py)."""
    for case in ref_runs["cases"]:
        B = case["batch"]
        s = O.Oracle(case["num_qubits"], B, seed=case["seed"])
        ops = np.array(case["ops"], np.int32).reshape(-1, 4)
        s.run(ops, np.array(case["params"], np.float32), np.array(case["forced"], np.uint8))
        for rid, (rb, db) in enumerate(case["records"]):
            res, det = s.record(rid)
            assert np.packbits(res.astype(np.uint8), bitorder="little").tolist() == rb, (case["name"], rid)
            assert np.packbits(det.astype(np.uint8), bitorder="little").tolist() == db, (case["name"], rid)
        h = hashlib.sha256()
        for a in s.tableau():
            h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
        assert h.hexdigest() == case["tableau_sha256"], case["name"]
        assert s.checksum() == case["checksum"]


def test_philox_known_answers(O):
    """Philox4x32-10 known-answer vectors published with Random123."""
    import ctypes as C
    L = O.lib()

    def ph(ctr, key):
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        out = (C.c_uint32 * 4)()
        L.ora_philox4x32_10(c, k, out)
        return list(out)

    assert ph([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert ph([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert ph([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]
