"""The C-ABI library loads without a GPU and exports every symbol the header declares."""
import ctypes
import os
import re

from sassena_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "sassena_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sass_[a-z_0-9]+)\s*\(", src)))


def test_header_lists_match_binding():
    assert header_functions() == sorted(abi.EXPORTS)


def test_library_exports_all_symbols():
    lib = abi.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.sass_version().startswith(b"sassena_gb300")
    assert lib.sass_status_name(3) == b"SASS_ERR_UNSUPPORTED"


def test_plan_create_rejects_bad_descriptors_without_gpu():
    lib = abi.load()
    h = ctypes.c_void_p()
    d = abi.PlanDesc(0, 0, 0, 0, 10, 0, 1, 0, None, 0)  # nf = 0
    assert lib.sass_plan_create(ctypes.byref(d), ctypes.byref(h)) == 1
    d = abi.PlanDesc(7, 0, 0, 0, 10, 10, 1, 0, None, 0)  # unknown scattering type
    assert lib.sass_plan_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert lib.sass_plan_create(None, ctypes.byref(h)) == 1
    # beyond the long-series transform: padded length above 2^20 (NF > 524,288)
    for scattering in (0, 1):
        d = abi.PlanDesc(scattering, 0, 0, 0, 10, 600000, 1, 0, None, 0)
        assert lib.sass_plan_create(ctypes.byref(d), ctypes.byref(h)) == 3
