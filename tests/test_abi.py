"""CPU tests of the C ABI library: it builds for sm_103a, loads, exports every function
include/orb/orb.h declares, and keeps the reference's 52-byte Cell layout."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "orb", "orb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(orb_[a-z_0-9]+)\s*\(", text)))


def test_header_matches_binding(engine):
    assert declared_functions() == sorted(engine.EXPORTS)


def test_library_exports_all_symbols(engine):
    lib = ctypes.CDLL(engine.LIB_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in orb.h but not exported"


def test_library_is_sm103a(engine):
    # nvcc records the embedded architectures; the build passes exactly one -gencode.
    assert engine.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.getsize(engine.LIB_PATH) > 0


def test_status_strings(engine):
    lib = engine.load()
    assert lib.orb_abi_version() == 3
    for code, text in engine.STATUS.items():
        assert lib.orb_status_string(code).decode() == text


def test_cell_layout(engine):
    dt = engine.CELL_DTYPE
    offs = {name: dt.fields[name][1] for name in dt.names}
    assert offs == {"id": 0, "nLeafCells": 4, "prevCutAxis": 8, "cutAxis": 12, "foundCut": 16,
                    "pad_": 17, "cutMarginLeft": 20, "cutMarginRight": 24, "lower": 28,
                    "upper": 40}
    assert dt.itemsize == 52


def test_tuning_layout_and_null_checks(engine):
    # orb_tuning: seven uint32 fields, no padding
    assert ctypes.sizeof(engine.Tuning) == 28
    lib = engine.load()
    t = engine.Tuning()
    assert lib.orb_get_tuning(None, ctypes.byref(t)) == 1
    assert lib.orb_set_tuning(None, ctypes.byref(t)) == 1
    assert lib.orb_autotune_batch(None, None, None, None, 0, None, 0, 0, 1, None, None) == 1


def test_invalid_arguments_without_device(engine):
    lib = engine.load()
    # null out-pointer is rejected before any CUDA call
    assert lib.orb_ctx_create(0, None, None) == 1
    assert lib.orb_ctx_destroy(None) == 1
    assert lib.orb_build(None, None, None, None, 0, 1, 0, None, None, None, None, None, 0, None) == 1


def test_no_device_reports_error(engine):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(engine.OrbError):
        engine.Context(0)
