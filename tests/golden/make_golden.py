"""Generate the golden fixtures under tests/golden/ (run in a container that
has the reference checked out; the outputs are committed).

1. reference_kat.json -- the known-answer vectors of the reference's own unit
   tests, read as text from plaquette_simulator/src/tests/Test_CliffordState.hpp
   (initial tableau, PauliProductPhase table, checksum fixture, the 110
   RowProductSign signs, the 110 RowMultiply checksums, MeasureDetermined
   outcomes, forced-bias checksums).
2. reference_runs.json -- outputs of the reference itself (its unmodified
   headers compiled on the project's Kokkos-API shim, oracle/_ref) for seeded
   circuits under forced random outcomes: per-record results / determined
   flags and a digest of the final tableau.
3. reference_circuits.json -- the same outputs of the reference for its own
   benchmark circuits (benchmarks/circuits.tar.gz, the line format of
   CliffordCircuit.hpp:32-66), each stored as the op table it parses to.
   The archive holds 59 text circuits; its member width_depth_4_10.circuit
   is itself a copy of the archive, not a circuit, and is left out.

Usage: python tests/golden/make_golden.py [--ref-src PATH]
(default: the checkout root of $REF_SRC, else the one oracle/Makefile names)
"""
from __future__ import annotations

import argparse
import ast
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "plaquette-simulator_gb300", "python"))

TEST_FILE = "plaquette_simulator/src/tests/Test_CliffordState.hpp"


def _blocks(text: str):
    """Map test-case name -> body text."""
    out = {}
    starts = [m for m in re.finditer(r'(?:TEMPLATE_)?TEST_CASE\("([^"]+)"', text)]
    for a, b in zip(starts, starts[1:] + [None]):
        out[a.group(1)] = text[a.start(): b.start() if b else len(text)]
    return out


def _literal(body: str, name: str):
    m = re.search(re.escape(name) + r"\s*=\s*(\{.*?\});", body, re.S)
    if not m:
        raise KeyError(name)
    src = m.group(1)
    src = re.sub(r"std::make_tuple\(([^)]*)\)", r"[\1]", src)
    src = src.replace("{", "[").replace("}", "]")
    return ast.literal_eval(src)


def _scalar(body: str, name: str):
    m = re.search(r"\b" + re.escape(name) + r"\s*=\s*([-0-9.]+)\s*;", body)
    return ast.literal_eval(m.group(1))


def kat(ref_root: str) -> dict:
    with open(os.path.join(ref_root, TEST_FILE)) as f:
        text = f.read()
    bl = _blocks(text)
    init = bl["CliffordStateKokkos::CheckInitialization"]
    phase = bl["Test PauliProductPhase"]
    cks = bl["Test Checksum"]
    rps = bl["CliffordStateKokkos::BatchRowProductSignFunctor"]
    rmu = bl["CliffordStateKokkos::BatchRowMultiplyFunctor"]
    mdet = bl["CliffordStateKokkos::BatchMeasureDeterminedFunctor"]
    mrand = bl["CliffordStateKokkos::MeasureRandom"]
    return {
        "source": TEST_FILE,
        "init_n3": {"x": _literal(init, "tableau_x_check"), "z": _literal(init, "tableau_z_check"),
                    "lines": "40-61"},
        "pauli_product_phase": {"paulis": _literal(phase, "paulis"), "expected": _literal(phase, "expected"),
                                "lines": "160-174"},
        "checksum_fixture": {"n": 5, "r": _literal(cks, "r_flat"), "x": _literal(cks, "x_flat"),
                             "z": _literal(cks, "z_flat"), "lines": "176-202"},
        "fixture5": {"n": 5, "r": _literal(rps, "r_flat"), "x": _literal(rps, "x_flat"),
                     "z": _literal(rps, "z_flat"), "lines": "212-222"},
        "row_product_sign": {"expected": _literal(rps, "expected"), "lines": "243-299"},
        "row_multiply_checksum": {"expected": _literal(rmu, "expected"), "lines": "377-433"},
        "measure_determined": {"expected": _literal(mdet, "expected_results"), "lines": "489"},
        "measure_random_bias": {"bias": [_scalar(mrand, "bias_1"), _scalar(mrand, "bias_2")],
                                "checksum": [_scalar(mrand, "check_sum_1"), _scalar(mrand, "check_sum_2")],
                                "lines": "513-542"},
    }


def tableau_digest(tab) -> str:
    h = hashlib.sha256()
    for a in tab:
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


def runs() -> dict:
    import oracle as O
    from plaquette_simulator import circuits as C

    O.build(ref=True)
    cases = []
    specs = [
        ("random_clifford_n6_b5", lambda: C.random_clifford(6, 80, seed=11), 5),
        ("random_clifford_n9_b70", lambda: C.random_clifford(9, 150, seed=12), 70),
        ("layered_w5_d6_b3", lambda: C.layered_circuit(5, 6, seed=13), 3),
        ("surface_d3_r2_p0_b17", lambda: C.surface_code_memory(3, 2, p=0.0), 17),
        ("surface_d3_r2_p05_b64", lambda: C.surface_code_memory(3, 2, p=0.05), 64),
        ("noisy_reset_n5_b9", None, 9),
    ]
    rng = np.random.default_rng(2024)
    for name, make, B in specs:
        if make is None:
            circ = C.random_clifford(5, 40, seed=14, measure_all=False)
            for q in range(5):
                circ.pauli1(q, 0.1, 0.2, 0.15)
            circ.pauli2(0, 3, [0.02 * (k + 1) for k in range(15)])
            for q in range(5):
                circ.r(q)
            circ.h(2)
            circ.cx(2, 4)
            for q in range(5):
                circ.m(q)
        else:
            circ = make()
        nm = circ.num_measurements()
        forced = rng.integers(0, 256, size=(max(nm, 1), (B + 7) // 8), dtype=np.uint8)
        seed = 1000 + len(cases)
        ref = O.Reference(circ.num_qubits, B, seed=seed)
        ref.run(circ.op_array(), circ.param_array(), forced)
        recs = []
        for rid in range(nm):
            res, det = ref.record(rid)
            recs.append([np.packbits(res.astype(np.uint8), bitorder="little").tolist(),
                         np.packbits(det.astype(np.uint8), bitorder="little").tolist()])
        cases.append({
            "name": name, "num_qubits": circ.num_qubits, "batch": B, "seed": seed,
            "ops": circ.op_array().reshape(-1).tolist(), "params": [float(v) for v in circ.param_array()],
            "forced": forced.tolist(), "records": recs,
            "tableau_sha256": tableau_digest(ref.tableau()), "checksum": int(ref.checksum()),
        })
    return {"generator": "reference headers on oracle/kokkos_shim (oracle/_ref/libplaquette_ref.so)",
            "cases": cases}


def bench_circuits(ref_root: str) -> dict:
    """The reference's benchmark circuits, run by the reference (oracle/_ref)
    and by the oracle on 70 shots (one full 64-shot word and a partial one)
    under seeded forced outcomes; the two must agree before anything is
    written."""
    import tarfile

    import oracle as O
    from plaquette_simulator import circuits as C

    O.build(ref=True)
    rng = np.random.default_rng(4242)
    cases = []
    with tarfile.open(os.path.join(ref_root, "benchmarks", "circuits.tar.gz")) as tf:
        for m in sorted(tf.getmembers(), key=lambda m: m.name):
            f = tf.extractfile(m)
            if f is None:
                continue
            raw = f.read()
            if raw[:2] == b"\x1f\x8b":  # the archive copy, not a circuit
                continue
            width = int(m.name.split("_")[2])
            circ = C.parse_text(raw.decode(), width)
            B = 70
            nm = circ.num_measurements()
            forced = rng.integers(0, 256, size=(max(nm, 1), (B + 7) // 8), dtype=np.uint8)
            seed = 7000 + len(cases)
            ref = O.Reference(width, B, seed=seed)
            ref.run(circ.op_array(), circ.param_array(), forced)
            ora = O.Oracle(width, B, seed=seed)
            ora.run(circ.op_array(), circ.param_array(), forced)
            assert all(np.array_equal(a, b) for a, b in zip(ref.tableau(), ora.tableau())), m.name
            recs = []
            for rid in range(nm):
                res, det = ref.record(rid)
                o_res, o_det = ora.record(rid)
                assert np.array_equal(res, o_res) and np.array_equal(det, o_det), (m.name, rid)
                recs.append([np.packbits(res.astype(np.uint8), bitorder="little").tolist(),
                             np.packbits(det.astype(np.uint8), bitorder="little").tolist()])
            cases.append({
                "name": m.name, "num_qubits": width, "batch": B, "seed": seed,
                "ops": circ.op_array().reshape(-1).tolist(), "params": [float(v) for v in circ.param_array()],
                "forced": forced.tolist(), "records": recs,
                "tableau_sha256": tableau_digest(ref.tableau()), "checksum": int(ref.checksum()),
            })
    return {"generator": "reference headers on oracle/kokkos_shim (oracle/_ref/libplaquette_ref.so), "
                         "benchmarks/circuits.tar.gz", "cases": cases}


def default_ref_root() -> str:
    src = os.environ.get("REF_SRC")
    if src:
        return os.path.abspath(os.path.join(src, "..", ".."))
    import subprocess
    out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref-root"], check=True,
                         capture_output=True, text=True)
    return out.stdout.strip()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=None, help="the reference checkout's root")
    args = ap.parse_args()
    if args.ref_src is None:
        args.ref_src = default_ref_root()
    with open(os.path.join(HERE, "reference_kat.json"), "w") as f:
        json.dump(kat(args.ref_src), f, indent=1)
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(runs(), f)
    with open(os.path.join(HERE, "reference_circuits.json"), "w") as f:
        json.dump(bench_circuits(args.ref_src), f, separators=(",", ":"))
    print("wrote reference_kat.json, reference_runs.json, reference_circuits.json in", HERE)


if __name__ == "__main__":
    main()
