"""channel_word, channel_word_surv and channel_word_est (ps_common.cuh, the
device's Pauli-channel samplers: survival products stepped one by one, binary
searched in a table, or walked to from a float estimate) compiled as host code with nvcc, against the oracle's
restatement (ora_channel_paulis) on the CPU: every shot of 12,000 words, one-
and two-qubit channels, totals from 0 to 1, bit for bit.  The GPU parity tests
check the device builds of the same functions."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "plaquette-simulator_gb300", "csrc")

PROGRAM = r"""
#include "ps_common.cuh"
#include <cmath>
#include <cstdio>
extern "C" void ora_channel_paulis(int64_t seed, uint64_t event, int64_t shot_base, int64_t batch, const float *p,
                                   int count, int32_t *out);
// the library's table (ps_gates.cu channel_thresholds), restated for this test
static void table(const float *p, int count, uint64_t *thr) {
    double cum = 0.0;
    for (int k = 0; k < count; ++k) {
        cum += (double)p[k];
        thr[k] = !(cum > 0.0) ? 0 : cum >= 1.0 ? (1ull << 32) : (uint64_t)std::floor(cum * 4294967296.0);
    }
    thr[count] = ps::channel_surv64(thr[count - 1]);
}
int main() {
    long bad = 0, hits = 0;
    const float p1[][3] = {{1e-3f, 1e-3f, 1e-3f}, {0.1f, 0.2f, 0.15f}, {0, 0, 0}, {0.5f, 0.3f, 0.2f}, {0, 1e-4f, 0}};
    float p15[15];
    for (int k = 0; k < 15; ++k) p15[k] = 0.004f * (k + 1);
    for (int c = 0; c < 6; ++c) {
        const float *p = c < 5 ? p1[c] : p15;
        const int count = c < 5 ? 3 : 15;
        uint64_t thr[16];
        table(p, count, thr);
        uint32_t surv[64];
        ps::channel_surv_table(thr[count - 1], surv);
        if (thr[count - 1] != 0 && surv[63] != thr[count]) ++bad;
        const ps::ChannelEst est = ps::channel_est_factors(thr[count - 1], count);
        for (uint64_t ev = 0; ev < 50; ++ev) {
            static int32_t o[64 * 40 + 1];
            ora_channel_paulis(12345 + c, ev, 128, 64 * 40, p, count, o);
            for (int64_t wd = 0; wd < 40; ++wd) {
                const ps::ChannelWord m = ps::channel_word(12345 + c, ev, 2 + wd, thr, count);
                const ps::ChannelWord m2 = ps::channel_word_surv(12345 + c, ev, 2 + wd, thr, count, surv);
                bad += m2.fxa != m.fxa || m2.fza != m.fza || m2.fxb != m.fxb || m2.fzb != m.fzb;
                const ps::ChannelWord m3 = ps::channel_word_est(12345 + c, ev, 2 + wd, thr, count, surv, est);
                bad += m3.fxa != m.fxa || m3.fza != m.fza || m3.fxb != m.fxb || m3.fzb != m.fzb;
                // a poor estimate (one that knows nothing) settles on the same outcomes
                const ps::ChannelWord m4 = ps::channel_word_est(12345 + c, ev, 2 + wd, thr, count, surv, ps::ChannelEst{0.0f, 0.0f});
                bad += m4.fxa != m.fxa || m4.fza != m.fza || m4.fxb != m.fxb || m4.fzb != m.fzb;
                for (int b = 0; b < 64; ++b) {
                    const int k = o[wd * 64 + b];
                    const int pa = count == 3 ? k : k >> 2, pb = count == 3 ? 0 : k & 3;
                    const u64 e[4] = {(u64)(pa == 1 || pa == 2), (u64)(pa == 2 || pa == 3), (u64)(pb == 1 || pb == 2),
                                      (u64)(pb == 2 || pb == 3)};
                    const u64 g[4] = {(m.fxa >> b) & 1, (m.fza >> b) & 1, (m.fxb >> b) & 1, (m.fzb >> b) & 1};
                    for (int t = 0; t < 4; ++t) bad += e[t] != g[t];
                    hits += k != 0;
                }
            }
        }
    }
    std::printf("%ld %ld\n", bad, hits);
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc")
def test_channel_word_matches_oracle_on_host(O, tmp_path):
    O.build(ref=False)
    so = O.ORACLE_SO
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "cw.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "cw"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, "-o", str(exe), str(src), so,
                    "-Xlinker", "-rpath", "-Xlinker", os.path.dirname(so)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    bad, hits = map(int, out.stdout.split())
    assert bad == 0 and hits > 10000
