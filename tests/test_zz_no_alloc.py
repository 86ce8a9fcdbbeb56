"""The allocation-free genomic-value entry point, for hosts that cannot let
the library allocate device memory.  It is called through the C ABI on
device buffers owned by the caller (here allocated by torch, outside the
call) and must give the same values as the allocating entry point, on two
calls in a row (the shared scratch keeps the previous call's contents)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, codes_d, freq_d, eff_d, pred_d, n, p, mu):
    return lib.sodagpu_compute_dgv_noalloc(n, p, C.c_void_p(codes_d.data_ptr()), n, C.c_void_p(freq_d.data_ptr()),
                                           float(mu), C.c_void_p(eff_d.data_ptr()), C.c_void_p(pred_d.data_ptr()),
                                           None)


def test_noalloc_dgv_matches_predict(gpu_lib):
    import torch

    import sodabayes_gb300 as sg
    rng = np.random.default_rng(17)
    n, p = 1237, 3001
    codes = rng.integers(0, 3, size=(n, p)).astype(np.int8)
    codes[:, 11] = 0                       # monomorphic column
    freq = codes.sum(axis=0) / (2.0 * n)
    dev = torch.device("cuda", 0)
    codes_d = torch.from_numpy(np.asfortranarray(codes).ravel(order="F")).to(dev)
    freq_d = torch.from_numpy(freq).to(dev)
    pred_d = torch.empty(n, dtype=torch.float64, device=dev)
    for call, mu in enumerate((3.25, -1.5)):
        eff = rng.standard_normal(p) * 0.05
        eff_d = torch.from_numpy(eff).to(dev)
        pred_d.fill_(np.nan)
        assert _call(gpu_lib, codes_d, freq_d, eff_d, pred_d, n, p, mu) == 0, call
        torch.cuda.synchronize()
        got = pred_d.cpu().numpy()
        want = sg.predict(codes=codes, freq=freq, mu=mu, effects=eff)
        assert np.all(np.isfinite(got))
        assert np.allclose(got, want, rtol=1e-12, atol=1e-12), call


def test_noalloc_rejects_oversized_input(gpu_lib):
    from sodabayes_gb300 import _abi
    too_many = 2 * 1024 * 1024 + 1
    rc = gpu_lib.sodagpu_compute_dgv_noalloc(too_many, 10, C.c_void_p(16), too_many, C.c_void_p(16), 0.0,
                                             C.c_void_p(16), C.c_void_p(16), None)
    assert rc == _abi.E_ARG
