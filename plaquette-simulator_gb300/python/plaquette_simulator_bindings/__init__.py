"""The module the reference's Python package imports.

The reference's ``plaquette_simulator/simulator.py:1`` is
``from plaquette_simulator_bindings import CliffordState``: a pybind11 module
(Bindings.cpp:11-31) over the Kokkos CliffordState<int>.  This package is a
drop-in for it over libps_gpu.so: the same class with the same constructor
(num_qubits, batch_size, seed, init_to_zero_state) and method names, so the
reference's Python package runs unchanged on top of it.

It does not import the ``plaquette_simulator`` package by name, because in
that setting the name belongs to the reference's own package: the
implementation next to it is loaded under a private name instead.
"""
import importlib.util
import os
import sys

_IMPL = __name__ + "._impl"
if _IMPL not in sys.modules:
    _dir = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "plaquette_simulator")
    _spec = importlib.util.spec_from_file_location(_IMPL, os.path.join(_dir, "__init__.py"),
                                                   submodule_search_locations=[_dir])
    _mod = importlib.util.module_from_spec(_spec)
    sys.modules[_IMPL] = _mod
    _spec.loader.exec_module(_mod)

from ._impl.simulator import CliffordState as _CliffordState  # noqa: E402


class CliffordState(_CliffordState):
    """Bindings.cpp:13-31: ``CliffordState(num_qubits, batch_size, seed,
    init_to_zero_state)`` (py::init<size_t, size_t, int, bool>) with
    get_num_qubits, get_batch_size, get_seed, reset_clifford_state,
    measure_qubit, get_kokkos_backend, get_measurement, apply_hadamard_gate,
    apply_control_not_gate, apply_control_phase_gate, apply_phase_gate,
    apply_pauli_x_gate, apply_pauli_z_gate and device_to_host."""

    def __init__(self, num_qubits: int, batch_size: int, seed: int, init_to_zero_state: bool):
        super().__init__(int(num_qubits), int(batch_size), int(seed), bool(init_to_zero_state))


# The member names of the reference's module (Bindings.cpp:15-31).
BINDING_METHODS = ("get_num_qubits", "get_batch_size", "get_seed", "reset_clifford_state", "measure_qubit",
                   "get_kokkos_backend", "get_measurement", "apply_hadamard_gate", "apply_control_not_gate",
                   "apply_control_phase_gate", "apply_phase_gate", "apply_pauli_x_gate", "apply_pauli_z_gate",
                   "device_to_host")

__all__ = ["CliffordState", "BINDING_METHODS"]
