"""A pin of the shared-x/z program builder (FrameBuilder, ps_frame.cpp): the
programs it emits for surface codes (d = 3, 5, 9) and random circuits (mixed
ops, many random measurements and resets, short row-major and long
column-major segments), before and after FrameBuilder::linearize, hashed
(FNV-1a over ops, rows, slot offsets, final x / z bits, launches).  The value
below was produced both by the current builder and by its predecessor that
scanned measurement columns in the row-major bits, so it also pins that
those two emit the same programs.  The device semantics of these programs
are what the GPU parity tests check; a deliberate change of the builder
changes this value."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "plaquette-simulator_gb300", "csrc")
PIN = "388c1cbcd31d2795"

PROGRAM = r"""
#include "ps_frame.h"
#include "plaquette_gpu.h"
#include <cstdio>
#include <cstdlib>
#include <vector>
using namespace ps;
static uint64_t H = 1469598103934665603ull;
static void hb(const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; ++i) { H ^= c[i]; H *= 1099511628211ull; }
}
template <class T> static void hv(const std::vector<T> &v) {
    const size_t n = v.size();
    hb(&n, 8);
    if (n) hb(v.data(), n * sizeof(T));
}
static void hp(const FrameProgram &p) {
    for (const FrameOp &o : p.ops) hb(&o, sizeof o);
    hv(p.tab); hv(p.slot_off); hv(p.xz); hv(p.rand_meas); hb(&p.entry_cap, 4);
    for (const auto &L : p.launches) {
        const uint32_t v[8] = {(uint32_t)L.seg, L.op0, L.op1, L.tab0, L.tab1, L.rand0, L.nrand, L.scratch};
        hb(v, sizeof v);
    }
}
int main(int argc, char **argv) {
    for (int k = 1; k + 1 < argc; k += 2) {
        const int64_t n = atoll(argv[k + 1]);
        FILE *f = fopen(argv[k], "rb");
        std::vector<int32_t> v;
        int32_t t;
        while (fread(&t, 4, 1, f) == 1) v.push_back(t);
        fclose(f);
        const size_t nops = v.size() / 4;
        for (int lin = 0; lin < 2; ++lin) {
            FrameBuilder fb(n);
            int seg = 0, meas = 0;
            for (size_t i = 0; i < nops;) {
                const int code = v[4 * i];
                if (code == PS_OP_M || code == PS_OP_R) {
                    fb.measure(v[4 * i + 1], meas++, code == PS_OP_R);
                    ++i;
                    continue;
                }
                size_t j = i;  // a segment: the run of ops up to the next measurement
                uint32_t nslots = 0;
                for (; j < nops && v[4 * j] != PS_OP_M && v[4 * j] != PS_OP_R; ++j)
                    nslots += v[4 * j] == PS_OP_PAULI1 || v[4 * j] == PS_OP_PAULI2;
                fb.begin_segment(seg++, nslots, j - i);
                uint32_t slot = 0;
                for (; i < j; ++i) {
                    const int c = v[4 * i], a = v[4 * i + 1], b = v[4 * i + 2];
                    if (c == PS_OP_PAULI1) fb.channel(a, -1, slot++);
                    else if (c == PS_OP_PAULI2) fb.channel(a, b, slot++);
                    else fb.gate(c, a, b);
                }
                fb.end_segment();
            }
            fb.finish();
            if (lin) fb.linearize(20000);
            hp(fb.prog);
        }
    }
    std::printf("%016llx\n", (unsigned long long)H);
    return 0;
}
"""


def _circuits():
    from plaquette_simulator import circuits as C
    from drivers import random_mixed_circuit
    out = [C.surface_code_memory(3, 3, p=1e-3), C.surface_code_memory(5, 5, p=1e-3),
           C.surface_code_memory(9, 3, p=1e-3)]
    for n, ops, seed in [(5, 300, 1), (17, 600, 2), (40, 900, 3), (70, 1500, 4)]:
        out.append(random_mixed_circuit(n, ops, seed=seed, flags=False))
    rng = C.SplitMix64(77)  # long segments (>= 64 ops) between measurement layers with random branches
    c = C.Circuit(30)
    for _ in range(6):
        for _ in range(120):
            k = rng.below(4)
            a, b = rng.below(30), rng.below(30)
            if k == 0:
                c.h(a)
            elif k == 1:
                c.s(a)
            elif k == 2 and a != b:
                c.cx(a, b)
            else:
                c.pauli1(a, 0.01, 0.01, 0.01)
        for q in range(30):
            if rng.below(2):
                c.m(q)
            else:
                c.r(q)
    out.append(c)
    return out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_frame_programs_pinned(tmp_path):
    args = []
    for k, circ in enumerate(_circuits()):
        path = tmp_path / f"c{k}.bin"
        np.ascontiguousarray(circ.op_array(), dtype=np.int32).tofile(path)
        args += [str(path), str(circ.num_qubits)]
    exe = tmp_path / "pin"
    src = tmp_path / "pin.cpp"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    str(src), os.path.join(CSRC, "ps_frame.cpp")], check=True)
    out = subprocess.run([str(exe)] + args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == PIN
