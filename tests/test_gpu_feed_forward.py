"""The scaled feed-forward workload of the bench (circuits.distillation_blocks:
the batched low-space S-state distillation of Test_CliffordState.hpp:675-741,
several blocks side by side, with H / S conditioned on each shot's own
measurements).  On the CPU the oracle shows the protocol's outcome; on the
GPU every record and the final tableau match the oracle in the fused
(per-shot) and plain forms."""
import numpy as np
import pytest


def _bits(words, shots):
    b = np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")
    return b[:, :shots].astype(np.int32)


def test_distillation_blocks_protocol_on_the_oracle(O):
    from plaquette_simulator import circuits as C
    blocks, shots = 4, 150
    c = C.distillation_blocks(blocks)
    assert c.num_qubits == 5 * blocks
    o = O.Oracle(c.num_qubits, shots, seed=1231232132)
    o.run(c.op_array(), c.param_array())
    nm = c.num_measurements()
    for k in range(nm - 4 * blocks, nm):
        res, det = o.record(k)
        assert np.all(det == 1) and np.all(res == (1 if k >= nm - blocks else 0)), k
    # the ancilla measurements are random (not determined) in every shot
    for k in range(7 * blocks):
        assert np.all(o.record(k)[1] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_distillation_blocks_match_oracle(ps, O, fused):
    from plaquette_simulator import circuits as C
    from plaquette_simulator.circuit import CompiledCircuit
    blocks, shots, seed = 6, 64 * 3 + 11, 77
    c = C.distillation_blocks(blocks)
    st = ps.CliffordState(c.num_qubits, shots, seed, True)
    cc = CompiledCircuit(c, st, fused=fused, graph=True)
    assert cc.stats["shared_xz"] == 0  # feed-forward: the per-shot plan
    cc.run(reset=True)
    nm = c.num_measurements()
    w = ((shots + 63) // 64 + 1) & ~1
    res, det = np.zeros((nm, w), np.uint64), np.zeros((nm, w), np.uint64)
    cc.copy_records_words(res, det)
    o = O.Oracle(c.num_qubits, shots, seed=seed)
    o.run(c.op_array(), c.param_array())
    gres, gdet = _bits(res, shots), _bits(det, shots)
    for k in range(nm):
        ores, odet = o.record(k)
        assert np.array_equal(gres[k], ores) and np.array_equal(gdet[k], odet), k
    x, z, r = st.device_to_host_numpy()
    ox, oz, orr = o.tableau()
    assert np.array_equal(x, ox) and np.array_equal(z, oz) and np.array_equal(r, orr)
