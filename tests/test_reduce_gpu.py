"""cns_reduce_state (stateless CFL dt and volume integrals on caller-owned device fields)
against the same formulas in numpy (FP64, 1e-12 relative)."""
import ctypes

import numpy as np
import pytest

from tests._util import smooth_random_state

pytestmark = pytest.mark.gpu


def _numpy_reduce(p, f, mu, dxv, dy, dz):
    r, u, v, w, e = f
    ien = e / r - 0.5 * (u * u + v * v + w * w)
    sos = np.sqrt(p.gam * (p.gam - 1) * ien)
    dx = dxv[None, None, :]
    conv = np.maximum((np.abs(u) + sos) / dx, np.maximum((np.abs(v) + sos) / dy, (np.abs(w) + sos) / dz))
    visc = np.maximum(mu / dx ** 2, np.maximum(mu / dy ** 2, mu / dz ** 2))
    dV = dx * dy * dz
    return np.array([min(1e5, np.min(p.cfl / np.maximum(conv, visc))), np.sum(r * dV), np.sum(r * w * dV),
                     np.sum(e * dV), np.sum((u * u + v * v + w * w) * dV)])


def device_inputs(p, seed=3):
    import torch
    f = smooth_random_state(p, seed=seed)
    mu = 0.001 + 0.0005 * np.abs(np.sin(np.arange(p.npoints))).reshape(p.shape)
    dxv = np.full(p.mx, p.Lx / p.mx) * (1.0 + 0.1 * np.cos(np.arange(p.mx)))
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in f + [mu]]
    return f, mu, dxv, dev, torch.from_numpy(dxv).cuda()


def test_reduce_state_matches_numpy(gpu_lib):
    import torch
    from cudanavierstokes_gb300.params import channel_params
    p = channel_params(24, 20, 28)
    f, mu, dxv, dev, ddxv = device_inputs(p)
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    dy, dz = p.Ly / p.my, p.Lz / p.mz
    rc = gpu_lib.cns_reduce_state(p.mx, p.my, p.mz, *[t.data_ptr() for t in dev], ddxv.data_ptr(), dy, dz, p.gam,
                                  p.cfl, out.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    ref = _numpy_reduce(p, f, mu, dxv, dy, dz)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12)


def test_reduce_state_rejects_bad_arguments(gpu_lib):
    assert gpu_lib.cns_reduce_state(0, 4, 4, *([None] * 7), 1.0, 1.0, 1.4, 0.5, None, None) == 1
