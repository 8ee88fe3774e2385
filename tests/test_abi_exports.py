"""The C ABI library loads without a GPU and exports every entry point the header declares."""
import ctypes
import os
import re

import leap_gb300 as lg
from leap_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "leap_gb300.h")


def declared_entry_points():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(leap_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "leap_calibrate" in names and "leap_set_metadata" in names and len(names) >= 10


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_abi.LIB_PATH)
    missing = [n for n in declared_entry_points() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert set(declared_entry_points()) <= set(_abi.SIGNATURES)


def test_no_device_gives_clean_error():
    # Without a GPU, context creation fails with a status, not a crash.
    import torch
    if torch.cuda.is_available():
        return
    try:
        lg.Context(0)
    except lg.LeapError as e:
        assert e.code == _abi.LEAP_ERR_CUDA
    else:
        raise AssertionError("expected LeapError without a GPU")


def test_synth_library_exports_its_header():
    from leap_gb300 import synth
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "leap_synth.h")).read(), flags=re.S)
    names = sorted(set(re.findall(r"\b(leap_[a-z0-9_]+)\s*\(", text)))
    assert names == ["leap_synth_fill_c64"]
    lib = synth._synth_lib()
    assert all(hasattr(lib, n) for n in names)
