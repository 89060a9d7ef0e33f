"""Per-op drivers shared by the parity tests: replay a circuit op table on
the GPU state (through the public CliffordState API, one C-ABI call per op)
or on a CPU engine (oracle / reference) with the same forced draws."""
import numpy as np

from plaquette_simulator import circuits as C


def run_ops_gpu(st, ops, params, forced_all=None, first_record=0):
    """Apply ops to a plaquette_simulator.CliffordState.  forced_all[k] are
    the packed bits of the k-th measurement (M or R) or None."""
    ops = np.asarray(ops, np.int32).reshape(-1, 4)
    k = 0
    for code, a, b, c in ops.tolist():
        f = None if forced_all is None or code not in (C.OP_M, C.OP_R) else forced_all[k]
        if code == C.OP_H:
            st.apply_hadamard_gate(a)
        elif code == C.OP_S:
            st.apply_phase_gate(a)
        elif code == C.OP_X:
            st.apply_pauli_x_gate(a)
        elif code == C.OP_Y:
            st.apply_pauli_y_gate(a)
        elif code == C.OP_Z:
            st.apply_pauli_z_gate(a)
        elif code == C.OP_CX:
            st.apply_control_not_gate(a, b)
        elif code == C.OP_CZ:
            st.apply_control_phase_gate(a, b)
        elif code == C.OP_M:
            st.measure_qubit(a, float(params[c]) if c >= 0 else 0.5, None, forced=f)
            k += 1
        elif code == C.OP_R:
            st.reset_qubit(a, forced=f)
            k += 1
        elif code == C.OP_PAULI1:
            st.pauli_channel_1(a, *[float(v) for v in params[c:c + 3]])
        elif code == C.OP_PAULI2:
            st.pauli_channel_2(a, b, [float(v) for v in params[c:c + 15]])
        elif code == C.OP_H_IF:
            st.apply_hadamard_gate_with_apply_flag(a, c + first_record)
        elif code == C.OP_S_IF:
            st.apply_phase_gate_with_apply_flag(a, c + first_record)
        else:
            raise ValueError(code)


def random_mixed_circuit(n, num_ops, seed, noise=True, flags=True):
    """Random circuit over every op kind the library supports."""
    rng = C.SplitMix64(seed)
    c = C.Circuit(n)
    nrec = 0
    for _ in range(num_ops):
        kind = rng.below(14 if (noise and flags) else 11)
        a = rng.below(n)
        b = rng.below(n)
        while n > 1 and b == a:
            b = rng.below(n)
        if kind == 0:
            c.h(a)
        elif kind == 1:
            c.s(a)
        elif kind == 2:
            c.x(a)
        elif kind == 3:
            c.y(a)
        elif kind == 4:
            c.z(a)
        elif kind in (5, 6) and n > 1:
            (c.cx if kind == 5 else c.cz)(a, b)
        elif kind == 7:
            c.m(a, bias=(0.5, 0.3, 1.0, 0.0)[rng.below(4)])
            nrec += 1
        elif kind == 8:
            c.r(a)
            nrec += 1
        elif kind == 9:
            c.h(a)
            c.cx(a, b) if n > 1 else c.s(a)
        elif kind == 10:
            c.m(a)
            nrec += 1
        elif kind == 11 and noise:
            c.pauli1(a, 0.1, 0.05, 0.2)
        elif kind == 12 and noise and n > 1:
            c.pauli2(a, b, [0.01 * (j + 1) for j in range(15)])
        elif kind == 13 and flags and nrec:
            rec = rng.below(nrec)
            (c.h_if if rng.below(2) else c.s_if)(a, rec)
        else:
            c.s(a)
    return c
