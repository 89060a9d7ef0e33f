"""CPU checks of the C ABI: the library builds for sm_103a, loads without a
GPU and exports every entry point declared in include/*.h (no compute call
is made here)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(ps_[a-z0-9_]+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_declared_symbols():
    import build as psbuild
    lib_path = psbuild.build()
    lib = ctypes.CDLL(lib_path)
    declared = _declared()
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def test_last_error_and_version_without_gpu():
    import build as psbuild
    lib = ctypes.CDLL(psbuild.build())
    lib.ps_version.restype = ctypes.c_char_p
    lib.ps_last_error.restype = ctypes.c_char_p
    assert lib.ps_version().startswith(b"plaquette-gb300")
    # A call on a null handle fails on the host, before any device work.
    assert lib.ps_h(None, ctypes.c_uint64(0)) == 1
    assert b"Error in Plaquette" in lib.ps_last_error()


def test_channel_probabilities_checked_on_the_host():
    """Pauli-channel probabilities are checked before the handle (and before
    any device work): each finite and in [0, 1].  A table summing past 1 is
    taken (its cumulative thresholds stop at 1).  A null handle with valid
    probabilities fails on the handle instead."""
    import build as psbuild
    lib = ctypes.CDLL(psbuild.build())
    lib.ps_last_error.restype = ctypes.c_char_p
    P3, P15 = ctypes.c_float * 3, ctypes.c_float * 15
    nan, inf = float("nan"), float("inf")
    for fn in (lib.ps_pauli_channel_1, lib.ps_pauli_channel_1_noalloc):
        for bad in ((nan, 0, 0), (-0.1, 0, 0), (0, 1.5, 0), (0, 0, inf), (0, -inf, 0)):
            assert fn(None, ctypes.c_uint64(0), P3(*bad)) == 1, bad
            assert b"probabilit" in lib.ps_last_error(), bad
        for good in ((0.0, 0.0, 0.0), (0.1, 0.2, 0.3), (1.0, 0.0, 0.0), (1 / 3, 1 / 3, 1 / 3), (0.5, 0.4, 0.2)):
            assert fn(None, ctypes.c_uint64(0), P3(*good)) == 1
            assert b"probabilit" not in lib.ps_last_error(), good
    bad15 = [0.0] * 15
    bad15[7] = nan
    assert lib.ps_pauli_channel_2(None, ctypes.c_uint64(0), ctypes.c_uint64(1), P15(*bad15)) == 1
    assert b"probabilit" in lib.ps_last_error()
    neg = [0.01] * 15
    neg[14] = -1e-3
    assert lib.ps_pauli_channel_2(None, ctypes.c_uint64(0), ctypes.c_uint64(1), P15(*neg)) == 1
    assert b"probability 14" in lib.ps_last_error()
    ok15 = [0.07] * 15  # sums to 1.05: taken
    assert lib.ps_pauli_channel_2(None, ctypes.c_uint64(0), ctypes.c_uint64(1), P15(*ok15)) == 1
    assert b"probabilit" not in lib.ps_last_error()


def test_product_has_no_oracle_dependency():
    """The CUDA library and the Python package never reference the oracle."""
    pkg = os.path.join(ROOT, "plaquette-simulator_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h", ".hpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "ps_oracle" not in text and "import oracle" not in text, f
