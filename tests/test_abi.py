"""The C-ABI libraries load and export every entry point include/*.h declares
(no device calls): the engine (rift_gb300.h) and the host layer
(rift_host.h)."""
import ctypes
import os
import re

from rift_gb300 import build as eb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="rift_gb300.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"\b(rift_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(eb.build())
    names = declared_symbols()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n


def test_host_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(eb.build_host())
    names = declared_symbols("rift_host.h")
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_product_has_no_cpu_fallback():
    """The package never loads the oracle: no reference to it in product code."""
    pkg = os.path.join(ROOT, "rift_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".hpp", ".cpp")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "rift_oracle" not in txt, f


def test_closure_library_exports_every_declared_symbol():
    eb.build()
    lib = ctypes.CDLL(eb.CLOSURE_LIB)
    names = declared_symbols("rift_closure.h")
    assert len(names) >= 6
    for n in names:
        assert hasattr(lib, n), n


def test_closure_struct_layouts_match_the_header():
    """The ctypes mirrors of rift_closure_src and rift_device_view have the
    C layout (offsets of the last members, total sizes)."""
    from rift_gb300 import capi, closure

    assert ctypes.sizeof(closure.Src) == 136
    assert closure.Src.samples.offset == 132
    assert closure.Src.sample_stride.offset == 96
    assert ctypes.sizeof(capi.DeviceView) == 104
    assert capi.DeviceView.kappa.offset == 96
