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

Usage: python tests/golden/make_golden.py [--ref-src PATH]
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default="/root/reference")
    args = ap.parse_args()
    with open(os.path.join(HERE, "reference_kat.json"), "w") as f:
        json.dump(kat(args.ref_src), f, indent=1)
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(runs(), f)
    print("wrote", os.path.join(HERE, "reference_kat.json"), os.path.join(HERE, "reference_runs.json"))


if __name__ == "__main__":
    main()
