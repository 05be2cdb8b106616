"""The C-ABI library loads, exports every symbol include/cns.h declares, and validates
parameters on the host (no compute without a GPU)."""
import ctypes
import os
import re

import pytest

from cudanavierstokes_gb300 import native
from cudanavierstokes_gb300.params import CnsParams, default_params, tgv_params

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(REPO, "include", fn)).read()
            names |= set(re.findall(r"^CNS_API\s+[\w\s\*]+?\b(cns_\w+)\s*\(", txt, flags=re.M))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"cns_create", "cns_run", "cns_copy_field", "cns_destroy", "cns_calc_rhs"} <= names


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in declared_symbols():
        assert hasattr(gpu_lib, name), name
    assert set(native.SIGNATURES) >= declared_symbols() - set()


def test_params_struct_layout_matches_default(gpu_lib):
    p = CnsParams()
    gpu_lib.cns_default_params(ctypes.byref(p))
    q = default_params()
    for k, v in q.as_dict().items():
        if k in ("mx", "my", "mz"):
            continue
        assert getattr(p, k) == pytest.approx(v), k


def test_parameter_validation(gpu_lib):
    assert gpu_lib.cns_check_params(ctypes.byref(tgv_params(16))) == 0
    for bad in (dict(stencil_size=5), dict(stencil_visc=0), dict(stencil_visc=4, stencil_size=3), dict(mx=4),
                dict(check_cfl=0), dict(precision=7), dict(scheme=9), dict(Ma=0.0),
                dict(boundary_layer=1, periodic_x=1)):
        p = tgv_params(16).copy(**bad)
        assert gpu_lib.cns_check_params(ctypes.byref(p)) == 1, bad
        assert gpu_lib.cns_last_error().decode()
    for prec in (0, 1, 2):   # FP64, FP32-RHS and pair mode
        assert gpu_lib.cns_check_params(ctypes.byref(tgv_params(16).copy(precision=prec))) == 0


def test_precision_constants_match_the_header():
    from cudanavierstokes_gb300 import params
    src = open(os.path.join(REPO, "include", "cns.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define CNS_(PREC_\w+)\s+(\d+)", src)}
    assert defs == {"PREC_FP64": params.PREC_FP64, "PREC_FP32_RHS": params.PREC_FP32_RHS,
                    "PREC_PAIR_RHS": params.PREC_PAIR_RHS}


def test_batch_rejects_the_pair_mode(gpu_lib):
    """Batches take FP64 or FP32-RHS; the argument check comes before any device call."""
    b = ctypes.c_void_p()
    assert gpu_lib.cns_batch_create(0, 2, 4, 4, 0, ctypes.byref(b)) == 1 and not b
    assert "CNS_PREC_FP32_RHS" in gpu_lib.cns_last_error().decode()


def test_largest_grids(gpu_lib):
    """Element offsets are 32-bit: a padded field must hold fewer than 2^31 elements. 1024^3
    (1.12e9 padded elements) is accepted, 1280^3 (2.16e9) is rejected with a message."""
    assert gpu_lib.cns_check_params(ctypes.byref(tgv_params(16).copy(mx=1024, my=1024, mz=1024))) == 0
    assert gpu_lib.cns_check_params(ctypes.byref(tgv_params(16).copy(mx=1280, my=1280, mz=1280))) == 1
    assert "2^31" in gpu_lib.cns_last_error().decode()


def test_create_fails_loudly_without_device(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = gpu_lib.cns_create(ctypes.byref(tgv_params(16)), 0, ctypes.byref(h))
    assert rc == 2 and not h
    assert "device" in gpu_lib.cns_last_error().decode()
