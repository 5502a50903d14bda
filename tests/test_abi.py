"""The C-ABI library builds, loads and exports every symbol the header declares
(no GPU needed: only the GPU-free entry points are called)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(fwant_\w+)\s*\(", txt, flags=re.M))
    return names


def test_header_declares_the_boundary():
    names = declared_symbols()
    for n in ("fwant_create", "fwant_destroy", "fwant_run", "fwant_set_media", "fwant_set_pml",
              "fwant_set_forces", "fwant_set_receivers", "fwant_get_seismo"):
        assert n in names


def test_library_exports_every_declared_symbol(native_lib):
    import fwant_gb300._lib as L
    missing = [n for n in declared_symbols() if not hasattr(native_lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in L.EXPORTS}
    assert declared_symbols() <= bound, declared_symbols() - bound


def test_gpu_free_entry_points(native_lib):
    import fwant_gb300 as fw
    assert native_lib.fwant_version().decode().startswith("fwant_gb300")
    # the reference runs whole 8-step blocks (exit test at the block start)
    assert fw.reference_steps(2000) == 2008
    assert fw.reference_steps(4000) == 4008
    assert fw.reference_steps(7) == 8
    assert fw.reference_steps(8) == 16


def test_create_rejects_bad_config(native_lib):
    import fwant_gb300 as fw
    with pytest.raises(fw.FwantError) as e:
        fw.Solver(4, 20, 20, 0.01)
    assert e.value.code in (1, 3)  # INVALID_ARG (or CUDA_ERROR where no device exists)
    # the configuration is validated before any device call
    for kw in (dict(storage=fw.STORAGE_FP64), dict(storage=7), dict(storage=fw.STORAGE_BF16, exact_arith=True),
               dict(storage=fw.STORAGE_FP16, exact_arith=True)):
        with pytest.raises(fw.FwantError) as e:
            fw.Solver(20, 20, 20, 0.01, **kw)
        assert e.value.code == 1, kw


def test_null_handles_are_rejected(native_lib):
    import ctypes as C
    import numpy as np
    out = np.zeros(9, np.float32)
    p = out.ctypes.data_as(C.POINTER(C.c_float))
    assert native_lib.fwant_max_abs(None, p) == 1
    assert native_lib.fwant_set_storage_scale(None, 1.0, 1.0) == 1
    assert native_lib.fwant_check(None) == 1
