"""Circuit representation, text format and seeded workload generators.

A circuit is a flat op table ``ops`` (int32 ``[k, 4]`` rows of
``(code, a, b, c)``) plus a float32 parameter table ``params``.  The same
encoding is consumed by the C-ABI (``ps_op`` in include/plaquette_gpu.h).

Codes (``a``/``b`` are qubits, ``c`` indexes ``params`` or names a record):

====  ======  ========================================================
 0    H       Hadamard on a
 1    S       phase gate on a
 2-4  X Y Z   Pauli gates on a
 5    CX      control a, target b
 6    CZ      control a, target b
 7    M       Z-basis measurement of a; bias = params[c] (c < 0: 0.5)
 8    R       reset of a: measurement into its own record, then X where 1
 9    PAULI1  Pauli channel on a; params[c:c+3] = (pX, pY, pZ)
10    PAULI2  two-qubit Pauli channel on (a, b); params[c:c+15] in the
              order IX IY IZ XI XX XY XZ YI YX YY YZ ZI ZX ZY ZZ
11    H_IF    Hadamard on a for shots whose record c is 1
12    S_IF    phase gate on a for shots whose record c is 1
====  ======  ========================================================

The text format follows the reference's circuit reader
(plaquette_simulator/src/CliffordCircuit.hpp:32-66): one op per line,
``NAME q0 q1 ...``, with NAME in {X, Y, Z, H, S, CX, CZ, M}; a multi-target
line applies the op to each target (CX / CZ to consecutive pairs).  This
module adds ``R``, and the Pauli channels ``E_PAULI px py pz q...`` and
``E_PAULI2 p1 ... p15 a b ...`` whose parameter counts the reference's reader
reserves (CliffordCircuit.hpp:44-56, commented out there).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

OP_H, OP_S, OP_X, OP_Y, OP_Z, OP_CX, OP_CZ, OP_M, OP_R, OP_PAULI1, OP_PAULI2, OP_H_IF, OP_S_IF = range(13)

OP_NAMES = {OP_H: "H", OP_S: "S", OP_X: "X", OP_Y: "Y", OP_Z: "Z", OP_CX: "CX", OP_CZ: "CZ", OP_M: "M",
            OP_R: "R", OP_PAULI1: "E_PAULI", OP_PAULI2: "E_PAULI2", OP_H_IF: "H_IF", OP_S_IF: "S_IF"}
GATE_CODES = (OP_H, OP_S, OP_X, OP_Y, OP_Z, OP_CX, OP_CZ, OP_M, OP_R)
RANDOM_CODES = (OP_M, OP_R, OP_PAULI1, OP_PAULI2)

_ONE_Q = {"H": OP_H, "S": OP_S, "X": OP_X, "Y": OP_Y, "Z": OP_Z, "M": OP_M, "R": OP_R}
_TWO_Q = {"CX": OP_CX, "CZ": OP_CZ}


@dataclass
class Circuit:
    """Op table + parameter table for ``num_qubits`` qubits."""

    num_qubits: int
    ops: List[Tuple[int, int, int, int]] = field(default_factory=list)
    params: List[float] = field(default_factory=list)
    _param_index: Dict[Tuple[float, ...], int] = field(default_factory=dict, repr=False)

    # -- building ------------------------------------------------------
    def _check(self, *qs: int) -> None:
        for q in qs:
            if not 0 <= q < self.num_qubits:
                raise ValueError(f"qubit {q} out of range for {self.num_qubits} qubits")

    def _param(self, values: Sequence[float]) -> int:
        key = tuple(float(np.float32(v)) for v in values)
        if key not in self._param_index:
            self._param_index[key] = len(self.params)
            self.params.extend(key)
        return self._param_index[key]

    def h(self, q): self._check(q); self.ops.append((OP_H, q, 0, 0))
    def s(self, q): self._check(q); self.ops.append((OP_S, q, 0, 0))
    def x(self, q): self._check(q); self.ops.append((OP_X, q, 0, 0))
    def y(self, q): self._check(q); self.ops.append((OP_Y, q, 0, 0))
    def z(self, q): self._check(q); self.ops.append((OP_Z, q, 0, 0))

    def cx(self, c, t):
        self._check(c, t)
        if c == t:
            raise ValueError("CX needs two distinct qubits")
        self.ops.append((OP_CX, c, t, 0))

    def cz(self, c, t):
        self._check(c, t)
        if c == t:
            raise ValueError("CZ needs two distinct qubits")
        self.ops.append((OP_CZ, c, t, 0))

    def m(self, q, bias: float = 0.5):
        self._check(q)
        self.ops.append((OP_M, q, 0, -1 if bias == 0.5 else self._param([bias])))

    def r(self, q): self._check(q); self.ops.append((OP_R, q, 0, -1))

    def pauli1(self, q, px: float, py: float, pz: float):
        self._check(q)
        self.ops.append((OP_PAULI1, q, 0, self._param([px, py, pz])))

    def pauli2(self, a, b, probs: Sequence[float]):
        self._check(a, b)
        if a == b or len(probs) != 15:
            raise ValueError("E_PAULI2 needs two distinct qubits and 15 probabilities")
        self.ops.append((OP_PAULI2, a, b, self._param(probs)))

    def depolarize1(self, q, p: float): self.pauli1(q, p / 3, p / 3, p / 3)
    def depolarize2(self, a, b, p: float): self.pauli2(a, b, [p / 15] * 15)

    def h_if(self, q, rec): self._check(q); self.ops.append((OP_H_IF, q, 0, rec))
    def s_if(self, q, rec): self._check(q); self.ops.append((OP_S_IF, q, 0, rec))

    # -- views -----------------------------------------------------------
    def op_array(self) -> np.ndarray:
        return np.asarray(self.ops, dtype=np.int32).reshape(-1, 4)

    def param_array(self) -> np.ndarray:
        return np.asarray(self.params if self.params else [0.0], dtype=np.float32)

    def arrays(self):
        """(op_array, param_array), converted once and reused while the
        circuit is unchanged (job submission hot path)."""
        key = (len(self.ops), len(self.params))
        cached = getattr(self, "_arrays", None)
        if cached is None or cached[0] != key:
            cached = (key, np.ascontiguousarray(self.op_array()), np.ascontiguousarray(self.param_array()))
            self._arrays = cached
        return cached[1], cached[2]

    def num_gates(self) -> int:
        """Gate applications per shot: H S X Y Z CX CZ M R (noise excluded)."""
        return sum(1 for o in self.ops if o[0] in GATE_CODES)

    def num_measurements(self) -> int:
        return sum(1 for o in self.ops if o[0] in (OP_M, OP_R))

    def num_records(self) -> int:
        return self.num_measurements()

    def __len__(self) -> int:
        return len(self.ops)

    def to_text(self) -> str:
        lines = []
        for code, a, b, c in self.ops:
            name = OP_NAMES[code]
            if code in (OP_CX, OP_CZ):
                lines.append(f"{name} {a} {b}")
            elif code == OP_PAULI1:
                lines.append(f"{name} " + " ".join(repr(v) for v in self.params[c:c + 3]) + f" {a}")
            elif code == OP_PAULI2:
                lines.append(f"{name} " + " ".join(repr(v) for v in self.params[c:c + 15]) + f" {a} {b}")
            elif code == OP_M and c >= 0:
                lines.append(f"MB {self.params[c]!r} {a}")
            elif code in (OP_H_IF, OP_S_IF):
                lines.append(f"{name} {c} {a}")
            else:
                lines.append(f"{name} {a}")
        return "\n".join(lines) + "\n"


def parse_text(text: str, num_qubits: int) -> Circuit:
    """Parse the line format of CliffordCircuit.hpp:32-66 (plus R, MB,
    E_PAULI, E_PAULI2, H_IF, S_IF).  Unknown names raise ValueError, like the
    reference's "Unsupported operation" error (CliffordCircuit.hpp:40-42).
    Blank lines are skipped.  Unlike the reference (which does not check),
    an out-of-range qubit or an odd CX/CZ target list raises ValueError."""
    circ = Circuit(num_qubits)
    for lineno, raw in enumerate(text.splitlines(), 1):
        tok = raw.split()
        if not tok:
            continue
        name, args = tok[0], tok[1:]
        try:
            if name in _ONE_Q:
                code = _ONE_Q[name]
                for a in args:
                    q = int(a)
                    circ._check(q)
                    circ.ops.append((code, q, 0, -1 if code in (OP_M, OP_R) else 0))
            elif name in _TWO_Q:
                qs = [int(a) for a in args]
                if len(qs) % 2:
                    raise ValueError(f"{name} needs an even number of targets")
                for k in range(0, len(qs), 2):
                    (circ.cx if name == "CX" else circ.cz)(qs[k], qs[k + 1])
            elif name == "MB":
                bias = float(args[0])
                for a in args[1:]:
                    circ.m(int(a), bias)
            elif name == "E_PAULI":
                p = [float(v) for v in args[:3]]
                for a in args[3:]:
                    circ.pauli1(int(a), *p)
            elif name == "E_PAULI2":
                p = [float(v) for v in args[:15]]
                qs = [int(a) for a in args[15:]]
                if len(qs) % 2:
                    raise ValueError("E_PAULI2 needs an even number of targets")
                for k in range(0, len(qs), 2):
                    circ.pauli2(qs[k], qs[k + 1], p)
            elif name in ("H_IF", "S_IF"):
                rec = int(args[0])
                for a in args[1:]:
                    (circ.h_if if name == "H_IF" else circ.s_if)(int(a), rec)
            else:
                raise ValueError(f"Unsupported operation: {name}")
        except (IndexError, ValueError) as e:
            raise ValueError(f"line {lineno}: {e}") from None
    return circ


# ---------------------------------------------------------------- generators
class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) for circuit generation."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def below(self, k: int) -> int:
        """Uniform integer in [0, k) by rejection (no modulo bias)."""
        lim = (1 << 64) - ((1 << 64) % k)
        while True:
            v = self.next()
            if v < lim:
                return v % k

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / (1 << 53))


def random_clifford(num_qubits: int = 64, num_gates: int = 1000, seed: int = 12345,
                    measure_all: bool = True) -> Circuit:
    """Random {H, S, CX} circuit then M on every qubit (the n=64 workload)."""
    rng = SplitMix64(seed)
    c = Circuit(num_qubits)
    for _ in range(num_gates):
        kind = rng.below(3)
        a = rng.below(num_qubits)
        if kind == 0:
            c.h(a)
        elif kind == 1:
            c.s(a)
        else:
            b = rng.below(num_qubits)
            while b == a:
                b = rng.below(num_qubits)
            c.cx(a, b)
    if measure_all:
        for q in range(num_qubits):
            c.m(q)
    return c


@dataclass
class SurfaceCodeLayout:
    distance: int
    data: List[Tuple[int, int]]
    x_anc: List[Tuple[int, int]]
    z_anc: List[Tuple[int, int]]
    index: Dict[Tuple[int, int], int]

    @property
    def num_qubits(self) -> int:
        return len(self.index)

    def ancillas(self) -> List[int]:
        return [self.index[p] for p in self.x_anc + self.z_anc]


# CX orders for the hook-avoiding schedule: X stabilizers visit their data
# qubits in a Z-shaped order, Z stabilizers in an N-shaped order.
_X_ORDER = [(1, 1), (1, -1), (-1, 1), (-1, -1)]
_Z_ORDER = [(1, 1), (-1, 1), (1, -1), (-1, -1)]


def surface_code_layout(d: int) -> SurfaceCodeLayout:
    """Rotated surface code of odd distance d: d*d data qubits on odd
    coordinates, d*d-1 ancillas on even coordinates; X-type plaquettes keep
    their weight-2 members on the top/bottom boundary, Z-type on left/right."""
    if d < 3 or d % 2 == 0:
        raise ValueError("distance must be odd and >= 3")
    data = [(2 * i + 1, 2 * j + 1) for j in range(d) for i in range(d)]
    dset = set(data)
    x_anc, z_anc = [], []
    for y in range(0, 2 * d + 1, 2):
        for x in range(0, 2 * d + 1, 2):
            nbrs = [(x + dx, y + dy) for dx, dy in ((1, 1), (1, -1), (-1, 1), (-1, -1)) if (x + dx, y + dy) in dset]
            is_x = ((x // 2) + (y // 2)) % 2 == 0
            interior = 0 < x < 2 * d and 0 < y < 2 * d
            if len(nbrs) == 4 and interior:
                (x_anc if is_x else z_anc).append((x, y))
            elif len(nbrs) == 2:
                on_tb = y in (0, 2 * d) and 0 < x < 2 * d
                on_lr = x in (0, 2 * d) and 0 < y < 2 * d
                if is_x and on_tb:
                    x_anc.append((x, y))
                elif not is_x and on_lr:
                    z_anc.append((x, y))
    index: Dict[Tuple[int, int], int] = {}
    for p in data + x_anc + z_anc:
        index[p] = len(index)
    return SurfaceCodeLayout(d, data, x_anc, z_anc, index)


def surface_code_memory(d: int, rounds: int | None = None, p: float = 1e-3) -> Circuit:
    """Rotated surface-code Z-memory: per round H on X-ancillas, four CX
    layers (hook-avoiding order), H on X-ancillas, M then R on every
    ancilla; then M on every data qubit.  With p > 0 every H is followed by a
    1-qubit depolarizing channel (p/3 each) and every CX by a 2-qubit one
    (p/15 each)."""
    lay = surface_code_layout(d)
    rounds = d if rounds is None else rounds
    c = Circuit(lay.num_qubits)
    xa = [lay.index[a] for a in lay.x_anc]
    anc = lay.ancillas()

    def h_layer():
        for q in xa:
            c.h(q)
            if p > 0:
                c.depolarize1(q, p)

    for _ in range(rounds):
        h_layer()
        for step in range(4):
            for (ax, ay) in lay.x_anc:
                dx, dy = _X_ORDER[step]
                dq = (ax + dx, ay + dy)
                if dq in lay.index:
                    c.cx(lay.index[(ax, ay)], lay.index[dq])
                    if p > 0:
                        c.depolarize2(lay.index[(ax, ay)], lay.index[dq], p)
            for (ax, ay) in lay.z_anc:
                dx, dy = _Z_ORDER[step]
                dq = (ax + dx, ay + dy)
                if dq in lay.index:
                    c.cx(lay.index[dq], lay.index[(ax, ay)])
                    if p > 0:
                        c.depolarize2(lay.index[dq], lay.index[(ax, ay)], p)
        h_layer()
        for q in anc:
            c.m(q)
        for q in anc:
            c.r(q)
    for (x, y) in lay.data:
        c.m(lay.index[(x, y)])
    return c


def surface_code_detectors(d: int, rounds: int | None = None):
    """Detectors and the logical observable of ``surface_code_memory(d,
    rounds)`` as lists of measurement indices (its record order: per round M
    then R of every ancilla, x_anc before z_anc; then M of every data qubit).

    Detectors: each Z-ancilla's round-1 outcome (fixed by |0...0>); every
    ancilla's outcome XOR its previous round's (rounds 2..); each Z-stabilizer
    rebuilt from the final data outcomes XOR its last ancilla outcome.  The
    observable is logical Z: the data qubits of the first row (y = 1), which
    meets every X-plaquette in 0 or 2 qubits.  Without noise every detector
    and the observable are 0 on every shot."""
    lay = surface_code_layout(d)
    rounds = d if rounds is None else rounds
    anc = lay.x_anc + lay.z_anc
    na = len(anc)
    nx = len(lay.x_anc)

    def m_anc(r, i):  # M of ancilla i in round r
        return r * 2 * na + i

    dpos = {p: k for k, p in enumerate(lay.data)}
    final = rounds * 2 * na
    dets = [[m_anc(0, i)] for i in range(nx, na)]
    for r in range(1, rounds):
        dets += [[m_anc(r, i), m_anc(r - 1, i)] for i in range(na)]
    for i in range(nx, na):
        ax, ay = anc[i]
        sup = [final + dpos[(ax + dx, ay + dy)] for dx, dy in ((1, 1), (1, -1), (-1, 1), (-1, -1))
               if (ax + dx, ay + dy) in dpos]
        dets.append(sup + [m_anc(rounds - 1, i)])
    observable = [final + dpos[(x, y)] for (x, y) in lay.data if y == 1]
    return dets, observable


def layered_circuit(width: int, depth: int, seed: int) -> Circuit:
    """Layers of one Pauli on every qubit, a ring of CX or CZ, then M on every
    qubit -- the shape of the reference's small benchmark circuits
    (benchmarks/circuits.tar.gz), drawn from a seeded generator."""
    rng = SplitMix64(seed)
    c = Circuit(width)
    for _ in range(depth):
        pauli = (c.x, c.y, c.z)[rng.below(3)]
        for q in range(width):
            pauli(q)
        two = c.cx if rng.below(2) == 0 else c.cz
        for q in range(width):
            two(q, (q + 1) % width)
        for q in range(width):
            c.m(q)
    return c


# The seven phasors of the low-space S-state distillation protocol
# (Test_CliffordState.hpp:675-741), over the block's data qubits 0..3.
DISTILLATION_PHASORS = ((0,), (1,), (2,), (0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))


def distillation_blocks(blocks: int) -> Circuit:
    """`blocks` independent copies of the batched low-space S-state
    distillation protocol (Test_CliffordState.hpp:675-741) side by side:
    block b holds data qubits 5b..5b+3 and ancilla 5b+4.  For each phasor
    every block entangles its ancilla with the phasor's data qubits, rotates
    and measures it, then undoes the rotation on every qubit involved with
    H / S gates conditioned on that measurement (H_IF, S_IF: per-shot
    feed-forward, so the circuit runs the per-shot plan).  The blocks step
    through the phasors together, so each phasor's measurements form one
    measurement phase.  Afterwards data qubits 0..2 of every block measure
    0 and qubit 3 (after S, H) measures 1, all determined, in every shot."""
    c = Circuit(5 * blocks)
    nrec = 0
    for phasor in DISTILLATION_PHASORS:
        for b in range(blocks):
            a = 5 * b + 4
            c.h(a)
            for k in phasor:
                c.cx(a, 5 * b + k)
            c.h(a)
            c.s(a)
            c.h(a)
        for b in range(blocks):
            c.m(5 * b + 4)
        for b in range(blocks):
            rec = nrec + b
            for q in [5 * b + k for k in phasor] + [5 * b + 4]:
                c.h_if(q, rec)
                c.s_if(q, rec)
                c.s_if(q, rec)
                c.h_if(q, rec)
        nrec += blocks
    for b in range(blocks):
        for k in range(3):
            c.m(5 * b + k)
    for b in range(blocks):
        c.s(5 * b + 3)
        c.h(5 * b + 3)
    for b in range(blocks):
        c.m(5 * b + 3)
    return c
