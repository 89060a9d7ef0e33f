"""Pipelined sampling (ps_circuit_copy_records_async / ps_circuit_wait_records):
two compiled copies of one circuit on one state, run in turn, each run's
records copied to pinned host memory while the next run computes, give the
records of the same number of consecutive runs of one circuit with
synchronous copies -- bit for bit, in both plans."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shared_xz", [True, False])
def test_pipelined_copies_match_consecutive_runs(ps, shared_xz):
    import torch
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    circ = C.surface_code_memory(5, 3, p=0.01)
    n, shots, seed, runs = circ.num_qubits, 64 * 9 + 5, 11, 5
    nm = circ.num_measurements()
    w = ((shots + 63) // 64 + 1) & ~1
    one = CompiledCircuit(circ, ps.CliffordState(n, shots, seed, True), fused=True, shared_xz=shared_xz)
    want = []
    for _ in range(runs):
        one.run(reset=True)
        res, det = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
        one.copy_records_words(res, det)
        want.append((res, det))
    st = ps.CliffordState(n, shots, seed, True)
    pair = [CompiledCircuit(circ, st, fused=True, shared_xz=shared_xz) for _ in range(2)]
    bufs = [[torch.zeros((nm, w), dtype=torch.int64, pin_memory=True) for _ in range(2)] for _ in range(runs)]
    for k in range(runs):
        cc = pair[k % 2]
        if k >= 2:
            cc.wait_records()
        cc.run(reset=True)
        cc.copy_records_async(bufs[k][0].numpy(), bufs[k][1].numpy())
    for cc in pair:
        cc.wait_records()
    for k in range(runs):
        got = [b.numpy().view(np.uint64) for b in bufs[k]]
        assert np.array_equal(got[0], want[k][0]), f"run {k}: results"
        assert np.array_equal(got[1], want[k][1]), f"run {k}: determined"
