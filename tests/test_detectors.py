"""Detectors and the logical observable of the surface-code memory circuit
(the step after the simulated path: XOR of ancilla records across rounds).
Definitions are checked on the CPU oracle -- without noise every detector
and the observable are 0 on every shot -- and the device extraction
(ps_circuit_detectors) against the XOR of the records read back."""
import numpy as np
import pytest


def _bits(words, shots):
    b = np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")
    return b[:, :shots].astype(np.int32)


@pytest.mark.parametrize("d,rounds", [(3, 3), (5, 2)])
def test_noiseless_detectors_are_zero_on_oracle(O, d, rounds):
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(d, rounds, p=0.0)
    dets, obs = C.surface_code_detectors(d, rounds)
    nz = (d * d - 1) // 2
    assert len(dets) == nz + (rounds - 1) * (d * d - 1) + nz
    assert len(obs) == d
    shots = 96
    o = O.Oracle(circ.num_qubits, shots, seed=5)
    o.run(circ.op_array(), circ.param_array())
    rec = np.stack([o.record(k)[0] for k in range(circ.num_measurements())])
    for dd in dets + [obs]:
        assert not np.bitwise_xor.reduce(rec[dd], axis=0).any()


def test_noise_fires_detectors_on_oracle(O):
    from plaquette_simulator import circuits as C
    circ = C.surface_code_memory(3, 3, p=0.05)
    dets, _ = C.surface_code_detectors(3, 3)
    o = O.Oracle(circ.num_qubits, 256, seed=9)
    o.run(circ.op_array(), circ.param_array())
    rec = np.stack([o.record(k)[0] for k in range(circ.num_measurements())])
    fired = sum(int(np.bitwise_xor.reduce(rec[dd], axis=0).sum()) for dd in dets)
    assert fired > 0


@pytest.mark.gpu
@pytest.mark.parametrize("p", [0.0, 5e-3])
def test_device_detectors_match_records(ps, p):
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    d, rounds, shots = 5, 4, 1000
    circ = C.surface_code_memory(d, rounds, p=p)
    dets, obs = C.surface_code_detectors(d, rounds)
    st = ps.CliffordState(circ.num_qubits, shots, 21, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.run(reset=True)
    nm = circ.num_measurements()
    w = ((shots + 63) // 64 + 1) & ~1
    res = np.zeros((nm, w), np.uint64)
    cc.copy_records_words(res, None)
    got = cc.detectors(dets + [obs])
    want = np.stack([np.bitwise_xor.reduce(res[dd], axis=0) for dd in dets + [obs]])
    assert np.array_equal(got, want)
    if p == 0.0:
        assert not _bits(got, shots).any()
    with pytest.raises(Exception):
        cc.detectors([[nm]])  # index past the last measurement
