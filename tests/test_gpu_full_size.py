"""The d=15 surface-code memory workload at full size (449 qubits, 15
rounds, p=1e-3, 16,384 shots) and shot ranges split over states.

The oracle cannot hold 16,384 shots of this circuit in its int32 layout
(53 GB), so parity at full size is pinned on two 64-shot slices: the first
and last shot words, simulated by the oracle with those global shot offsets
(its draws are keyed by global shot like the GPU's).  The records of every
measurement and the final tableau words of those shots must agree bit for
bit; size-independent properties cover the rest (determined flags of the
deterministic rounds, a replay with the same seed)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pack_word(a):
    """Oracle int32 [64, ...] 0/1 -> one uint64 per trailing index (bit s = shot s)."""
    b = np.packbits(np.asarray(a, dtype=bool), axis=0, bitorder="little")  # [8, ...]
    return np.ascontiguousarray(np.moveaxis(b, 0, -1)).view(np.uint64)[..., 0]


def _bits(words, shots):
    b = np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")
    return b[:, :shots].astype(np.int32)


@pytest.fixture(scope="module")
def full_run(ps):
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    circ = C.surface_code_memory(15, 15, p=1e-3)
    S = 16384
    st = ps.CliffordState(circ.num_qubits, S, 12345, True)
    cc = CompiledCircuit(circ, st, fused=True, graph=True)
    cc.run(reset=True)
    nm = circ.num_measurements()
    w = ((S + 63) // 64 + 1) & ~1
    res = np.zeros((nm, w), np.uint64)
    det = np.zeros_like(res)
    cc.copy_records_words(res, det)
    return circ, st, cc, res, det


@pytest.mark.parametrize("word", [0, 255])
def test_full_size_slice_matches_oracle(full_run, O, word):
    circ, st, cc, res, det = full_run
    o = O.Oracle(circ.num_qubits, 64, seed=12345, shot_base=64 * word)
    o.run(circ.op_array(), circ.param_array())
    gres = _bits(res[:, word:word + 1], 64)
    gdet = _bits(det[:, word:word + 1], 64)
    for k in range(circ.num_measurements()):
        ores, odet = o.record(k)
        assert np.array_equal(gres[k], ores), f"record {k} results differ"
        assert np.array_equal(gdet[k], odet), f"record {k} determined differ"
    gx, gz, gr = st.tableau_words(word, 1)
    ox, oz, orr = o.tableau()
    assert np.array_equal(gx[:, :, 0], _pack_word(ox)), "x words differ"
    assert np.array_equal(gz[:, :, 0], _pack_word(oz)), "z words differ"
    assert np.array_equal(gr[:, 0], _pack_word(orr)), "r words differ"


def test_full_size_properties(full_run):
    circ, st, cc, res, det = full_run
    S = st.get_batch_size()
    # Rounds 2..15 measure stabilizers that are already fixed: every shot is
    # determined (records: M and R of the 224 ancillas per round, then the
    # 225 data qubits).
    per_round = 2 * (15 * 15 - 1)
    assert circ.num_measurements() == 15 * per_round + 15 * 15
    dbits = _bits(det, S)
    assert dbits[per_round:15 * per_round].all(), "a mid-circuit ancilla measurement was random"
    # Replaying with the same seed and event base reproduces every record.
    st.set_event_counter(0)
    cc.run(reset=True)
    res2 = np.zeros_like(res)
    det2 = np.zeros_like(det)
    cc.copy_records_words(res2, det2)
    assert np.array_equal(res, res2) and np.array_equal(det, det2)


def test_split_states_reproduce_one_state(ps):
    """A job's shots split over two states with shot offsets (one per GPU in
    a multi-GPU run) give exactly the records of one state."""
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    circ = C.surface_code_memory(5, 3, p=5e-3)
    nm = circ.num_measurements()

    def records(shots, offset):
        st = ps.CliffordState(circ.num_qubits, shots, 77, True)
        st.set_shot_offset(offset)
        cc = CompiledCircuit(circ, st, fused=True, graph=True)
        cc.run(reset=True)
        w = ((shots + 63) // 64 + 1) & ~1
        res = np.zeros((nm, w), np.uint64)
        det = np.zeros_like(res)
        cc.copy_records_words(res, det)
        return _bits(res, shots), _bits(det, shots)

    whole = records(640, 0)
    left = records(384, 0)
    right = records(256, 384)
    assert np.array_equal(np.concatenate([left[0], right[0]], axis=1), whole[0])
    assert np.array_equal(np.concatenate([left[1], right[1]], axis=1), whole[1])
