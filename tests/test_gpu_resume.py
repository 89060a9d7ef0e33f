"""Packed snapshot / resume (ps_copy_tableau_words, ps_load_tableau_words):
a state parked between two circuits as packed words plus its event
counter, and resumed in a fresh state, continues exactly as the state run
straight through -- records and final tableau bit for bit.  The import path
of the reference is HostToDevice (CliffordState.hpp:207-231) in its int32
layout; this one moves 1 bit per (row, qubit, shot) instead of 32."""
import numpy as np
import pytest

from drivers import random_mixed_circuit

pytestmark = pytest.mark.gpu


def _records(cc, nm, shots):
    w = ((shots + 63) // 64 + 1) & ~1
    res, det = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
    cc.copy_records_words(res, det)
    return res, det


@pytest.mark.parametrize("fused", [True, False])
def test_resume_continues_like_the_run_through(ps, fused):
    from plaquette_simulator.circuit import CompiledCircuit
    n, shots, seed = 12, 64 * 5 + 13, 99
    first = random_mixed_circuit(n, 300, seed=61)
    second = random_mixed_circuit(n, 300, seed=62)
    through = ps.CliffordState(n, shots, seed, True)
    CompiledCircuit(first, through, fused=fused).run(reset=True)
    snap = through.snapshot()
    b1 = CompiledCircuit(second, through, fused=fused)
    b1.run(reset=False)
    resumed = ps.CliffordState.resume(snap)
    assert resumed.event_counter() == snap["events"]
    b2 = CompiledCircuit(second, resumed, fused=fused)
    b2.run(reset=False)
    nm = second.num_measurements()
    for a, b in zip(_records(b1, nm, shots), _records(b2, nm, shots)):
        assert np.array_equal(a, b)
    for a, b in zip(through.device_to_host_numpy(), resumed.device_to_host_numpy()):
        assert np.array_equal(a, b)


def test_resume_by_shot_ranges(ps):
    """Words loaded range by range (two halves, r only in the second call
    for the first half) give the same state as one load."""
    n, shots = 7, 64 * 8
    src = ps.CliffordState(n, shots, 5, True)
    for q in range(n):
        src.apply_hadamard_gate(q)
    src.apply_control_not_gate(0, 3)
    src.measure_qubit(3)
    src.apply_phase_gate(5)
    x, z, r = src.tableau_words(0, src.words())
    dst = ps.CliffordState(n, shots, 5, True)
    h = src.words() // 2
    dst.load_tableau_words(0, x[..., :h], z[..., :h], None)
    dst.load_tableau_words(h, x[..., h:], z[..., h:], r[..., h:])
    dst.load_tableau_words(0, None, None, r[..., :h])
    for a, b in zip(src.device_to_host_numpy(), dst.device_to_host_numpy()):
        assert np.array_equal(a, b)
    from plaquette_simulator import _lib
    with pytest.raises(_lib.PlaquetteError) as e:
        dst.load_tableau_words(src.words(), x[..., :1], None, None)
    assert e.value.status == _lib.PS_E_RANGE
