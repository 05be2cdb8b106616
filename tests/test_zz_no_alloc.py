"""The allocation-free reduction entry point against the allocating one, through the C ABI.

cns_reduce_state_noalloc serves callers that may not allocate device memory (memory owned
by another allocator or a fixed budget, loops that must not block in the allocator): its
partial sums live in a fixed device array shared by every call. This file is collected last so that a run which
stops at the first failure has run every other test before it; it also passes on its own
in a fresh process (the array's device address is looked up on the first call).
"""
import ctypes

import numpy as np
import pytest

from cudanavierstokes_gb300.params import channel_params, tgv_params
from tests._util import smooth_random_state

pytestmark = pytest.mark.gpu


def _device_case(p, seed):
    import torch
    f = smooth_random_state(p, seed=seed)
    mu = 0.001 + 0.0005 * np.abs(np.sin(np.arange(p.npoints) * 0.37)).reshape(p.shape)
    dxv = np.full(p.mx, p.Lx / p.mx) * (1.0 + 0.1 * np.cos(np.arange(p.mx)))
    fields = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in f + [mu]]
    return fields, torch.from_numpy(dxv).cuda()


def _call(lib, name, p, fields, dxv, out, stream):
    fn = getattr(lib, name)
    return fn(p.mx, p.my, p.mz, *[t.data_ptr() for t in fields], dxv.data_ptr(), p.Ly / p.my, p.Lz / p.mz, p.gam,
              p.cfl, out.data_ptr(), ctypes.c_void_p(stream))


def test_noalloc_matches_allocating_entry_point_two_calls(gpu_lib):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row with different sizes and inputs: the shared scratch keeps the
    # first call's partials, which must not leak into the second result
    for p, seed in ((channel_params(24, 20, 64), 5), (tgv_params(16).copy(my=12, mz=40), 6)):
        fields, dxv = _device_case(p, seed)
        ref = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
        got = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(gpu_lib, "cns_reduce_state", p, fields, dxv, ref, stream) == 0
        assert _call(gpu_lib, "cns_reduce_state_noalloc", p, fields, dxv, got, stream) == 0
        torch.cuda.synchronize()
        a, b = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


def test_noalloc_rejects_too_many_planes(gpu_lib):
    import torch
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    one = torch.ones(1, dtype=torch.float64, device="cuda")
    ptr = one.data_ptr()
    rc = gpu_lib.cns_reduce_state_noalloc(4, 4, 4097, *([ptr] * 7), 1.0, 1.0, 1.4, 0.5, out.data_ptr(), None)
    assert rc == 1
    assert "4096" in gpu_lib.cns_last_error().decode()
