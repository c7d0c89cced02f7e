"""The allocation-free observables entry point (isg_cont_observables_static).

It serves callers that cannot call cudaMalloc, such as code whose device memory
all comes from its own pool, so it keeps its block partials in a fixed device
array. This test calls it through the C ABI on lattices that the test owns, and
checks it against the allocating path (isg_cont_measure). The allocating path
sums in exact fixed point and this one in compensated FP32 with an FP64 combine,
so the two differ by rounding and the tolerance is 2e-6 per bond, as in
tests/test_gpu_continuous.py. It makes two calls in a row
on different lattices, because the second call reuses the partials the first one
left behind. The file is named to run last, and the test also passes on its own
in a fresh process."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_entry(pkg):
    f = pkg.lib().isg_cont_observables_static
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("nc,L,R", [(3, 16, 3), (2, 12, 4)])
def test_static_observables_match_measure(gpu, nc, L, R):
    import torch
    entry = _static_entry(gpu)
    b = gpu.ContinuousBatch([L], R, nc, seed=1234)
    b.set_temperatures([1.4 + 0.05 * r for r in range(R)])
    out = torch.zeros(R * 10, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        b.sweep(5 + 10 * call, 0.5, 2)
        e, m, hb = b.measure()
        spins = np.stack([b.get_spins(0, r).reshape(-1) for r in range(R)]).astype(np.float32)
        d_spins = torch.from_numpy(spins).cuda()
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = entry(d_spins.data_ptr(), L, nc, R, 1.0, out.data_ptr(), stream)
        assert rc == 0, gpu.lib().isg_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(R, 10)
        tol = 2e-6 * 3 * L ** 3
        assert np.all(np.abs(got[:, 0] - e) < tol)
        assert np.all(np.abs(got[:, 1:4] - m) < tol)
        assert np.all(np.abs(got[:, 4:10] - hb) < tol)


def test_static_observables_reject_oversize(gpu):
    import torch
    entry = _static_entry(gpu)
    d = torch.zeros(8, dtype=torch.float32, device="cuda")
    out = torch.zeros(10, dtype=torch.float64, device="cuda")
    # 17 lattices of 128^3 sites need 17 * 2048 > 16384 partial blocks
    rc = entry(d.data_ptr(), 128, 3, 17, 1.0, out.data_ptr(), None)
    assert rc == -1 and b"fixed scratch" in gpu.lib().isg_last_error()
