"""The shared-x/z sign program's measurement phases as linear maps
(FrameBuilder::linearize, ps_frame.cpp): on the CPU, a model of the sign
kernel runs the program before and after the rewrite on the same random
signs, channel flips and random outcomes, and every record, determined flag
and final sign must agree bit for bit.  Random circuits (gates, channels,
M and R with many random branches), several register sizes, and shared-memory
budgets small enough to cut the runs at every place they can be cut."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "plaquette-simulator_gb300", "csrc")

PROGRAM = r"""
#include "ps_frame.h"
#include "plaquette_gpu.h"
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>
using namespace ps;

static uint64_t mix(uint64_t x) {  // SplitMix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Result { std::map<int, std::pair<uint64_t, uint64_t>> rec; std::vector<uint64_t> R; };

// frame_kernel's ops on one 64-shot word: channel ops XOR keyed random
// masks into their rows, random outcomes are keyed by (launch, index).
static Result run(const FrameProgram &p, int64_t n, uint64_t key) {
    const int64_t W = 2 * n + 1;
    std::vector<uint64_t> R(W);
    for (int64_t i = 0; i < W; ++i) R[i] = mix(key ^ (0x1000 + i));
    Result out;
    int noise_no = 0;
    for (size_t li = 0; li < p.launches.size(); ++li) {
        const auto &L = p.launches[li];
        std::vector<uint64_t> s(W + 1 + kWinRows + L.nrand, 0ull);
        for (int64_t i = 0; i < W; ++i) s[i] = R[i];
        for (uint32_t j = 0; j < L.nrand; ++j) s[kLinRand0(W) + j] = mix(key ^ (li << 20) ^ (j + 7));
        uint64_t last = 0;
        const std::vector<uint32_t> &T = p.tab;
        for (uint32_t oi = L.op0; oi < L.op1; ++oi) {
            const FrameOp o = p.ops[oi];
            const uint32_t kind = o.kind & 0xFFu;
            if (kind == F_NOISE) {
                const uint64_t h = mix(key ^ (0xABCD00000ull + noise_no++));
                for (int t = 0; t < 5; ++t) s[mix(h + t) % W] ^= mix(h ^ (t + 99));
            } else if (kind == F_WINDOW) {
                std::vector<uint64_t> acc(o.len);
                for (uint32_t j = 0; j < o.len; ++j) {
                    const uint32_t *rc = &T[o.off + kWinRec * j];
                    acc[j] = (rc[1] & 1u) ? ~0ull : 0ull;
                    for (uint32_t t = 0; t < kWinRows; ++t) acc[j] ^= s[rc[2 + t]];
                    out.rec[(int)rc[0]] = {acc[j], ~0ull};
                }
                s[2 * n] = acc[o.len - 1];
                for (uint32_t j = 0; j < o.len; ++j)
                    for (uint32_t t = 0; t < kWinRows; ++t) s[T[o.off + kWinRec * j + 2 + kWinRows + t]] ^= acc[j];
                last = acc[o.len - 1];
            } else if (kind == F_MEAS_DET) {
                uint64_t acc = 0;
                for (uint32_t t = o.off; t < o.off + o.len; ++t) acc ^= s[T[t]];
                if (o.kind >> 8) acc = ~acc;
                out.rec[o.arg] = {acc, ~0ull};
                s[2 * n] = acc;
                last = acc;
            } else if (kind == F_MEAS_RAND) {
                const uint64_t v = s[kLinRand0(W) + (o.kind >> 8)];
                const uint32_t q = T[o.off];
                const uint64_t rpv = s[q + n];
                s[q] = rpv;
                s[q + n] = v;
                out.rec[o.arg] = {v, 0ull};
                for (uint32_t t = o.off + 1; t < o.off + o.len; ++t)
                    s[T[t] & 0x7FFFFFFFu] ^= rpv ^ ((T[t] >> 31) ? ~0ull : 0ull);
                last = v;
            } else if (kind == F_RESET_X || kind == F_FLIP) {
                const uint64_t m = kind == F_RESET_X ? last : ~0ull;
                for (uint32_t t = o.off; t < o.off + o.len; ++t) s[T[t]] ^= m;
            } else if (kind == F_LINEAR) {
                const uint32_t *Lr = &T[o.off];
                const uint32_t nrec = Lr[0], nrow = Lr[1], nlast = Lr[2], nout = nrec + nrow + nlast;
                const uint32_t *dst = Lr + 4, *beg = dst + nout, *term = beg + nout + 1;
                std::vector<uint64_t> nv(nrow + nlast);
                for (uint32_t j = 0; j < nout; ++j) {
                    uint64_t v = (dst[j] & kLinConst) ? ~0ull : 0ull;
                    for (uint32_t t = beg[j]; t < beg[j + 1]; ++t) v ^= s[term[t]];
                    if (j < nrec) out.rec[(int)(dst[j] & kLinIndex)] = {v, (dst[j] & kLinDet) ? ~0ull : 0ull};
                    else nv[j - nrec] = v;
                }
                for (uint32_t j = 0; j < nrow; ++j) s[dst[nrec + j] & kLinIndex] = nv[j];
                if (nlast) last = nv[nrow];
            } else {
                std::printf("FAIL unknown op kind %u\n", kind);
                std::exit(1);
            }
        }
        for (int64_t i = 0; i < W; ++i) R[i] = s[i];
    }
    out.R = R;
    return out;
}

static FrameBuilder build(int64_t n, uint64_t seed, int rounds) {
    FrameBuilder fb(n);
    uint64_t st = seed;
    auto rnd = [&](uint64_t m) { st = mix(st); return m ? st % m : 0; };
    int seg = 0, meas = 0;
    for (int r = 0; r < rounds; ++r) {
        if (rnd(4) != 0) {  // a segment of gates and channels
            const int ng = 1 + (int)rnd(3 * n + 3);
            std::vector<int> ops(ng);
            uint32_t nslots = 0;
            for (int g = 0; g < ng; ++g) { ops[g] = (int)rnd(9); nslots += ops[g] >= 7; }
            fb.begin_segment(seg++, nslots, (size_t)ng);
            uint32_t slot = 0;
            for (int g = 0; g < ng; ++g) {
                const int64_t a = (int64_t)rnd(n);
                int64_t b = (int64_t)rnd(n);
                if (n > 1 && b == a) b = (a + 1) % n;
                const int code = ops[g];
                if (code == 7) fb.channel(a, -1, slot++);
                else if (code == 8) fb.channel(a, n > 1 ? b : -1, slot++);
                else if ((code == PS_OP_CX || code == PS_OP_CZ) && n < 2) fb.gate(PS_OP_H, a, -1);
                else fb.gate(code, a, b);
            }
            fb.end_segment();
        }
        const int nm = (int)rnd(2 * n + 2);
        for (int m = 0; m < nm; ++m) fb.measure((int64_t)rnd(n), meas++, rnd(3) == 0);
    }
    fb.finish();
    return fb;
}

int main() {
    int checked = 0, linear_ops = 0, kept = 0;
    const int64_t sizes[] = {1, 2, 3, 5, 9, 17, 40};
    const uint32_t budgets[] = {2, 3, 5, 17, 1u << 20};
    for (int64_t n : sizes)
        for (uint64_t seed = 1; seed <= 6; ++seed)
            for (uint32_t budget : budgets) {
                FrameBuilder a = build(n, seed * 1000 + n, 12);
                FrameBuilder b = build(n, seed * 1000 + n, 12);
                b.linearize(budget);
                for (const FrameOp &o : b.prog.ops) {
                    linear_ops += (o.kind & 0xFFu) == F_LINEAR;
                    kept += (o.kind & 0xFFu) != F_LINEAR && (o.kind & 0xFFu) != F_NOISE;
                }
                for (const auto &L : b.prog.launches)
                    for (uint32_t i = L.op0; i < L.op1; ++i) {
                        const FrameOp &o = b.prog.ops[i];
                        if ((o.kind & 0xFFu) == F_LINEAR && (o.off < L.tab0 || o.off + o.len > L.tab1)) {
                            std::printf("FAIL n=%lld: F_LINEAR outside the launch's tab range\n", (long long)n);
                            return 1;
                        }
                        if ((o.kind & 0xFFu) == F_LINEAR && b.prog.tab[o.off + 1] + b.prog.tab[o.off + 2] > L.scratch) {
                            std::printf("FAIL n=%lld: scratch too small\n", (long long)n);
                            return 1;
                        }
                    }
                for (uint64_t key = 0; key < 3; ++key) {
                    const Result ra = run(a.prog, n, key * 77 + seed), rb = run(b.prog, n, key * 77 + seed);
                    if (ra.rec != rb.rec || ra.R != rb.R) {
                        std::printf("FAIL n=%lld seed=%llu budget=%u key=%llu\n", (long long)n,
                                    (unsigned long long)seed, budget, (unsigned long long)key);
                        return 1;
                    }
                    ++checked;
                }
            }
    std::printf("OK %d linear %d kept %d\n", checked, linear_ops, kept);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_linearized_phases_equal_op_by_op(tmp_path):
    src = tmp_path / "lin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "lin"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    str(src), os.path.join(CSRC, "ps_frame.cpp")], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    words = out.stdout.split()
    assert words[0] == "OK"
    assert int(words[3]) > 0 and int(words[5]) > 0, out.stdout  # both linear runs and ops kept on their own
