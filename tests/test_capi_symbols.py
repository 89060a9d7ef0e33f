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


def test_product_has_no_oracle_dependency():
    """The CUDA library and the Python package never reference the oracle."""
    pkg = os.path.join(ROOT, "plaquette-simulator_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h", ".hpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "ps_oracle" not in text and "import oracle" not in text, f
