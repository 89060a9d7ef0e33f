"""The allocation-free Pauli channel (ps_pauli_channel_1_noalloc).

Callers that cannot allocate device memory mid-run -- a host that gave the
whole device to its own memory pool up front, or a process held to a strict
memory budget -- use this entry point instead of ps_pauli_channel_1.  It must
give exactly the same tableau as the allocating entry point, call after call,
while keeping its scratch in a fixed array inside the library.

This file is collected last on purpose, and each test builds its own states,
so it passes both alone in a fresh process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _prepare(ps, n, shots, seed):
    st = ps.CliffordState(n, shots, seed, True)
    for q in range(n):
        st.apply_hadamard_gate(q)
        if q % 2:
            st.apply_phase_gate(q)
    for q in range(n - 1):
        st.apply_control_not_gate(q, q + 1)
    return st


def test_noalloc_channel_matches_allocating_entry_point(ps):
    from plaquette_simulator import _lib
    L = _lib.load()
    n, shots, seed = 6, 64 * 37 + 5, 4242
    ref = _prepare(ps, n, shots, seed)
    new = _prepare(ps, n, shots, seed)
    calls = [(2, (0.2, 0.1, 0.3)), (5, (0.0, 0.45, 0.05))]  # two calls in a row
    for q, probs in calls:
        p = np.asarray(probs, dtype=np.float32)
        _lib.check(L.ps_pauli_channel_1(ref.handle, q, p.ctypes.data_as(C.c_void_p)))
        _lib.check(L.ps_pauli_channel_1_noalloc(new.handle, q, p.ctypes.data_as(C.c_void_p)))
        new.synchronize()
        for a, b in zip(ref.device_to_host_numpy(), new.device_to_host_numpy()):
            assert np.array_equal(a, b)  # bit-exact: integer tableau data
        assert ref.event_counter() == new.event_counter()


def test_noalloc_channel_at_the_size_limit(ps):
    """The largest batch it takes: 64 * 8192 shots, exactly 8192 shot-words,
    so the outcome masks fill the whole array behind the threshold slots."""
    from plaquette_simulator import _lib
    L = _lib.load()
    n, shots, seed = 1, 64 * 8192, 777
    ref = _prepare(ps, n, shots, seed)
    new = _prepare(ps, n, shots, seed)
    for probs in ((0.3, 0.2, 0.1), (0.05, 0.0, 0.6)):
        p = np.asarray(probs, dtype=np.float32)
        _lib.check(L.ps_pauli_channel_1(ref.handle, 0, p.ctypes.data_as(C.c_void_p)))
        _lib.check(L.ps_pauli_channel_1_noalloc(new.handle, 0, p.ctypes.data_as(C.c_void_p)))
        new.synchronize()
        for a, b in zip(ref.device_to_host_numpy(), new.device_to_host_numpy()):
            assert np.array_equal(a, b)
        assert ref.event_counter() == new.event_counter()


def test_noalloc_channel_rejects_oversized_batch(ps):
    from plaquette_simulator import _lib
    L = _lib.load()
    st = ps.CliffordState(1, 64 * 8192 + 1, 1, True)
    p = np.asarray([0.1, 0.1, 0.1], dtype=np.float32)
    rc = L.ps_pauli_channel_1_noalloc(st.handle, 0, p.ctypes.data_as(C.c_void_p))
    assert rc == _lib.PS_E_ARG
    assert b"allocation-free limit" in L.ps_last_error()
