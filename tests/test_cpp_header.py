"""The C++ drop-in header (include/plaquette/CliffordState.hpp): it compiles
on CPU, and on a GPU a program written against the reference's
Plaquette::CliffordState API runs the reference's protocol tests
(Test_CliffordState.hpp:66-158, :544-572) and its feed-forward tests
(:635-741, flag gates fed with GetMeasurement(id).measurement_results_device)
through libps_gpu.so, plus GetX/GetZ/GetR into DeviceToDevice (:168-174,
:268-274)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <plaquette/CliffordState.hpp>
#include <cstdio>
#include <cstdlib>
#include <vector>

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
    {   // PhaseKickbackBatched as the reference writes it (Test_CliffordState.hpp:635-672)
        CliffordState<int> kokkos_state_1(2, 2);
        kokkos_state_1.ApplyHadamardGate(1);
        kokkos_state_1.ApplyPhaseGate(1);
        kokkos_state_1.ApplyHadamardGate(0);
        kokkos_state_1.ApplyControlNotGate(0, 1);
        auto measurement_id = kokkos_state_1.MeasureQubit(1);
        auto &measurement = kokkos_state_1.GetMeasurement(measurement_id);
        REQUIRE(kokkos_state_1.GetMeasurement(measurement_id, 0).value().second == 0);
        REQUIRE(kokkos_state_1.GetMeasurement(measurement_id, 1).value().second == 0);
        kokkos_state_1.ApplyPhaseGateWithApplyFlag(0, *measurement.measurement_results_device);
        kokkos_state_1.ApplyPhaseGateWithApplyFlag(0, *measurement.measurement_results_device);
        kokkos_state_1.ApplyPhaseGate(0);
        kokkos_state_1.ApplyHadamardGate(0);
        measurement_id = kokkos_state_1.MeasureQubit(0);
        for (size_t k = 0; k < 2; ++k) {
            auto r = kokkos_state_1.GetMeasurement(measurement_id, k);
            REQUIRE(r.value().second == 1 && r.value().first == 1);
        }
    }
    {   // S-state distillation, low space, batched (Test_CliffordState.hpp:675-741)
        const size_t batch_size = 100;
        CliffordState<int> sim(5, batch_size, 1231232132);
        std::vector<std::vector<int>> phasors = {{0}, {1}, {2}, {0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
        const int anc = 4;
        for (const auto &phasor : phasors) {
            sim.ApplyHadamardGate(anc);
            for (int k : phasor) sim.ApplyControlNotGate(anc, k);
            sim.ApplyHadamardGate(anc);
            sim.ApplyPhaseGate(anc);
            sim.ApplyHadamardGate(anc);
            auto measurement_id = sim.MeasureQubit(anc);
            auto &measurement = sim.GetMeasurement(measurement_id);
            REQUIRE(measurement.qubit_measured == (size_t)anc);
            for (size_t b = 0; b < batch_size; b++) REQUIRE(sim.GetMeasurement(measurement_id, b).value().second == 0);
            measurement.CopyToHost();
            REQUIRE(measurement.measurement_results_host.size() == batch_size);
            for (size_t b = 0; b < batch_size; b++)
                REQUIRE(measurement.measurement_results_host[b] == sim.GetMeasurement(measurement_id, b).value().first);
            for (int k : phasor) {
                sim.ApplyHadamardGateWithApplyFlag(k, *measurement.measurement_results_device);
                sim.ApplyPhaseGateWithApplyFlag(k, *measurement.measurement_results_device);
                sim.ApplyPhaseGateWithApplyFlag(k, *measurement.measurement_results_device);
                sim.ApplyHadamardGateWithApplyFlag(k, *measurement.measurement_results_device);
            }
            sim.ApplyHadamardGateWithApplyFlag(anc, *measurement.measurement_results_device);
            sim.ApplyPhaseGateWithApplyFlag(anc, *measurement.measurement_results_device);
            sim.ApplyPhaseGateWithApplyFlag(anc, *measurement.measurement_results_device);
            sim.ApplyHadamardGateWithApplyFlag(anc, *measurement.measurement_results_device);
        }
        for (int k = 0; k < 3; ++k) {
            auto measurement_id = sim.MeasureQubit(k);
            for (size_t b = 0; b < batch_size; b++) {
                auto result = sim.GetMeasurement(measurement_id, b);
                REQUIRE(result.value().first == 0 && result.value().second == 1);
            }
        }
        sim.ApplyPhaseGate(3);
        sim.ApplyHadamardGate(3);
        auto measurement_id = sim.MeasureQubit(3);
        for (size_t b = 0; b < batch_size; b++) {
            auto result = sim.GetMeasurement(measurement_id, b);
            REQUIRE(result.value().first == 1 && result.value().second == 1);
        }
        bool out_of_range = false;
        try { sim.GetMeasurement(1000); } catch (const Plaquette::Exception &) { out_of_range = true; }
        REQUIRE(out_of_range);
    }
    {   // the copy constructor's path: GetX/GetZ/GetR into DeviceToDevice
        CliffordState<int> a(4, 130, 9);
        a.ApplyHadamardGate(0); a.ApplyControlNotGate(0, 1); a.ApplyPhaseGate(2); a.ApplyHadamardGate(3);
        a.MeasureQubit(1);
        CliffordState<int> b(4, 130, 9, false);
        b.DeviceToDevice(a.GetX(), a.GetZ(), a.GetR());
        REQUIRE(b.CheckSum() == a.CheckSum());
        auto [ax, az, ar] = a.DeviceToHost();
        auto [bx, bz, br] = b.DeviceToHost();
        REQUIRE(ax == bx && az == bz && ar == br);
        REQUIRE(a.GetX().rows == 9 && a.GetX().cols == 4 && a.GetR().cols == 1);
        CliffordState<int> small(3, 130);
        bool mismatch = false;
        try { small.DeviceToDevice(a.GetX(), a.GetZ(), a.GetR()); } catch (const Plaquette::Exception &) { mismatch = true; }
        REQUIRE(mismatch);
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
