"""The ``plaquette_simulator_bindings`` module: the name the reference's
Python package imports its CliffordState from (plaquette_simulator/
simulator.py:1, Bindings.cpp:11).  On CPU it imports and offers every member
the pybind11 module binds; on a GPU a package shaped like the reference's
(``plaquette_simulator`` whose simulator imports from
plaquette_simulator_bindings) runs the reference's Python test
(tests/test_clifford_state.py) and a feed-forward check on top of it."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PYDIR = os.path.join(ROOT, "plaquette-simulator_gb300", "python")


def test_bindings_module_offers_the_bound_members():
    sys.path.insert(0, PYDIR)
    import plaquette_simulator_bindings as b
    for name in b.BINDING_METHODS:
        assert callable(getattr(b.CliffordState, name, None)), name
    import inspect
    params = list(inspect.signature(b.CliffordState.__init__).parameters)
    assert params == ["self", "num_qubits", "batch_size", "seed", "init_to_zero_state"]


# A package laid out like the reference's (its __init__ re-exports the
# simulator's CliffordState; the simulator takes it from the bindings).
REF_SHAPED_INIT = "from .simulator import CliffordState\n"
REF_SHAPED_SIMULATOR = "from plaquette_simulator_bindings import CliffordState\n"

CHECK = textwrap.dedent("""
    import plaquette_simulator as ps
    assert ps.__file__.startswith(REFDIR), ps.__file__   # the reference-shaped package, not ours
    # tests/test_clifford_state.py: TestInitialization
    state = ps.CliffordState(3, 10, 0, True)
    assert state.get_num_qubits() == 3 and state.get_batch_size() == 10 and state.get_seed() == 0
    x, z, r = state.device_to_host()
    assert len(x) == 10 * 7 * 3 and len(z) == 10 * 7 * 3 and len(r) == 10 * 7
    # |0...0>: destabilizers X_i, stabilizers Z_i (CliffordState.hpp:97-139)
    for b in range(10):
        for i in range(3):
            for j in range(3):
                assert x[(b * 7 + i) * 3 + j] == (i == j) and z[(b * 7 + 3 + i) * 3 + j] == (i == j)
    # Bell pair over the batch through the bound members
    state.apply_hadamard_gate(0)
    state.apply_control_not_gate(0, 1)
    m0 = state.measure_qubit(0, 0.5, None)
    m1 = state.measure_qubit(1, 0.5, None)
    for b in range(10):
        r0, r1 = state.get_measurement(m0, b), state.get_measurement(m1, b)
        assert r0[1] == 0 and r1[1] == 1 and r0[0] == r1[0]
    assert state.get_measurement(m1 + 1, 0) is None and state.get_measurement(m0, 10) is None
    state.apply_phase_gate(2); state.apply_pauli_x_gate(2); state.apply_pauli_z_gate(2)
    state.apply_control_phase_gate(1, 2)
    assert isinstance(state.get_kokkos_backend(), str)
    state.reset_clifford_state()
    m2 = state.measure_qubit(2, 0.5, None)
    assert all(state.get_measurement(m2, b) == (0, 1) for b in range(10))
    print("OK")
""")


def test_reference_shaped_package_imports_the_bindings(tmp_path):
    """Without a GPU: with a reference-shaped ``plaquette_simulator`` first on
    the path, its CliffordState is the bindings' class, and the bindings
    never bound the name ``plaquette_simulator`` to this repository's package."""
    import build as psbuild
    psbuild.build()
    pkg = tmp_path / "plaquette_simulator"
    pkg.mkdir()
    (pkg / "__init__.py").write_text(REF_SHAPED_INIT)
    (pkg / "simulator.py").write_text(REF_SHAPED_SIMULATOR)
    code = textwrap.dedent(f"""
        import sys
        import plaquette_simulator as ps
        import plaquette_simulator_bindings as b
        assert ps.__file__.startswith({str(tmp_path)!r}), ps.__file__
        assert ps.CliffordState is b.CliffordState
        assert sys.modules["plaquette_simulator"] is ps
        print("OK")
    """)
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(tmp_path), PYDIR]))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120,
                         cwd=str(tmp_path))
    assert out.returncode == 0 and "OK" in out.stdout, out.stdout + out.stderr


@pytest.mark.gpu
def test_reference_shaped_package_runs_on_the_bindings(gpu_lib, tmp_path):
    pkg = tmp_path / "plaquette_simulator"
    pkg.mkdir()
    (pkg / "__init__.py").write_text(REF_SHAPED_INIT)
    (pkg / "simulator.py").write_text(REF_SHAPED_SIMULATOR)
    code = f"REFDIR = {str(tmp_path)!r}\n" + CHECK
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(tmp_path), PYDIR]))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300,
                         cwd=str(tmp_path))
    assert out.returncode == 0 and "OK" in out.stdout, out.stdout + out.stderr
