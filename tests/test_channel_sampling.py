"""Pauli-channel sampling (ora_channel_paulis in the oracle; channel_word in
ps_common.cuh draws the same bits on the device, which the GPU parity tests
check): per word, the gaps between hit shots are drawn from the survival
products, and each hit picks its Pauli from the channel's conditional
distribution.  Here, on the CPU, the outcomes must have the distribution of
independent per-shot draws: every Pauli at its probability, and the number
of hits in a 64-shot word Binomial(64, p).  Both are chi-square tests at a
fixed seed, with a 1e-4 false-alarm level."""
import ctypes as C

import numpy as np
import pytest
from scipy import stats


def _paulis(O, seed, event, shot_base, batch, p):
    L = O.lib()
    p = np.ascontiguousarray(p, dtype=np.float32)
    out = np.zeros(batch + 1, dtype=np.int32)
    L.ora_channel_paulis(seed, event, shot_base, batch, p.ctypes.data_as(C.c_void_p), len(p),
                         out.ctypes.data_as(C.c_void_p))
    return out[:batch]


@pytest.mark.parametrize("p", [
    [0.01, 0.02, 0.03],
    [0.2, 0.1, 0.3],
    [0.0, 0.05, 0.0],
    [0.004 * (k + 1) for k in range(15)],
])
def test_pauli_frequencies(O, p):
    counts = np.zeros(len(p) + 1)
    for ev in range(40):
        k = _paulis(O, 7, ev, 0, 64 * 400, p)
        counts += np.bincount(k, minlength=len(p) + 1)
    probs = np.array([1.0 - sum(p)] + list(p))
    keep = probs > 0
    assert counts[~keep].sum() == 0  # a zero-probability Pauli never appears
    chi2, pval = stats.chisquare(counts[keep], counts.sum() * probs[keep])
    assert pval > 1e-4, (counts, chi2)


@pytest.mark.parametrize("ptot", [0.003, 0.05, 0.4])
def test_hits_per_word_binomial(O, ptot):
    p = [ptot / 3] * 3
    hits = []
    for ev in range(20):
        k = _paulis(O, 11, ev, 0, 64 * 2000, p).reshape(-1, 64)
        hits.append((k != 0).sum(axis=1))
    hits = np.concatenate(hits)
    pmf = stats.binom.pmf(np.arange(65), 64, ptot)
    # pool the tails so that every expected count is at least 5
    exp = pmf * len(hits)
    obs = np.bincount(hits, minlength=65).astype(float)
    lo = int(np.argmax(np.cumsum(exp) >= 5))
    hi = 64 - int(np.argmax(np.cumsum(exp[::-1]) >= 5))
    e = np.concatenate([[exp[:lo + 1].sum()], exp[lo + 1:hi], [exp[hi:].sum()]])
    o = np.concatenate([[obs[:lo + 1].sum()], obs[lo + 1:hi], [obs[hi:].sum()]])
    chi2, pval = stats.chisquare(o, e * o.sum() / e.sum())
    assert pval > 1e-4, (o, e, chi2)


def test_words_are_independent_of_the_batch_split(O):
    """Outcomes are keyed by global shot: one call over 640 shots equals
    calls over pieces starting at any shot (as on several GPUs)."""
    p = [0.05, 0.1, 0.02]
    whole = _paulis(O, 3, 9, 0, 640, p)
    parts = np.concatenate([_paulis(O, 3, 9, a, b - a, p) for a, b in [(0, 64), (64, 100), (100, 640)]])
    assert np.array_equal(whole, parts)
    assert whole.any()
