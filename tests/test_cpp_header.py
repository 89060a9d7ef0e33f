"""The C++ drop-in header (include/plaquette/CliffordState.hpp): it compiles
on CPU, and on a GPU a program written against the reference's
Plaquette::CliffordState API runs the reference's protocol tests
(Test_CliffordState.hpp:66-158, :544-572) through libps_gpu.so."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <plaquette/CliffordState.hpp>
#include <cstdio>
#include <cstdlib>

#define REQUIRE(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); std::exit(1); } } while (0)

using Plaquette::CliffordState;

int main() {
    {   // Measure0: H S S H |0> = |1>, deterministic
        CliffordState<int> s(1, 1);
        s.ApplyHadamardGate(0); s.ApplyPhaseGate(0); s.ApplyPhaseGate(0); s.ApplyHadamardGate(0);
        s.MeasureQubit(0);
        auto r = s.GetMeasurement(0, 0);
        REQUIRE(r.has_value() && r->first == 1 && r->second == 1);
        REQUIRE(!s.GetMeasurement(1, 0).has_value());
    }
    {   // EPR over a batch
        CliffordState<int> s(2, 100, 11);
        s.ApplyHadamardGate(0);
        s.ApplyControlNotGate(0, 1);
        size_t a = s.MeasureQubit(0), b = s.MeasureQubit(1);
        for (size_t k = 0; k < 100; ++k) {
            auto ra = s.GetMeasurement(a, k), rb = s.GetMeasurement(b, k);
            REQUIRE(ra->second == 0 && rb->second == 1 && ra->first == rb->first);
        }
    }
    {   // PhaseKickbackBatched with flag gates (Test_CliffordState.hpp:635-672)
        CliffordState<int> s(2, 2);
        s.ApplyHadamardGate(1); s.ApplyPhaseGate(1); s.ApplyHadamardGate(0); s.ApplyControlNotGate(0, 1);
        size_t id = s.MeasureQubit(1);
        s.ApplyPhaseGateWithApplyFlag(0, id);
        s.ApplyPhaseGateWithApplyFlag(0, id);
        s.ApplyPhaseGate(0); s.ApplyHadamardGate(0);
        id = s.MeasureQubit(0);
        for (size_t k = 0; k < 2; ++k) REQUIRE(s.GetMeasurement(id, k)->first == 1);
    }
    {   // host round trip and checksum
        CliffordState<int> s(3, 2);
        auto [x, z, r] = s.DeviceToHost();
        CliffordState<int> t(x, z, r, 3, 2);
        REQUIRE(t.CheckSum() == s.CheckSum());
        CliffordState<int> c(t);
        REQUIRE(c.CheckSum() == s.CheckSum());
    }
    bool threw = false;
    try { CliffordState<int> s(2, 1); s.ApplyHadamardGate(5); } catch (const Plaquette::Exception &e) { threw = true; }
    REQUIRE(threw);
    std::printf("OK\n");
    return 0;
}
"""


def _write(tmp_path):
    src = tmp_path / "prog.cpp"
    src.write_text(PROGRAM)
    return src


def test_header_compiles(tmp_path):
    src = _write(tmp_path)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_header_program_runs(gpu_lib, tmp_path):
    src = _write(tmp_path)
    libdir = os.path.join(ROOT, "plaquette-simulator_gb300", "lib")
    exe = tmp_path / "prog"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lps_gpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and "OK" in out.stdout, out.stdout + out.stderr
