"""The allocation-free genomic-value entry point, for hosts that cannot let
the library allocate device memory.  It is called through the C ABI on
device buffers owned by the caller (here allocated by torch, outside the
call) and must give the same values as the allocating entry point, on two
calls in a row (the shared scratch keeps the previous call's contents).

Cases: codes with leading dimension nind on the default stream; a padded
leading dimension with the call enqueued on a caller's stream; more than
65,536 individuals (fewer column splits than sodagpu_predict, so the last
bits may differ: 1e-12 relative); codes outside 0..2, which count as 1 here
and must match sodagpu_predict on the codes with those entries set to 1; and
sizes beyond the scratch maximum, rejected before anything is launched."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, codes_d, ldg, freq_d, eff_d, pred_d, n, p, mu, stream=None):
    return lib.sodagpu_compute_dgv_noalloc(n, p, C.c_void_p(codes_d.data_ptr()), ldg, C.c_void_p(freq_d.data_ptr()),
                                           float(mu), C.c_void_p(eff_d.data_ptr()), C.c_void_p(pred_d.data_ptr()),
                                           None if stream is None else C.c_void_p(stream.cuda_stream))


def _device_codes(codes, ldg):
    """(n, p) int8 codes as a device buffer with leading dimension ldg (padding filled with 7)."""
    import torch
    n, p = codes.shape
    buf = np.full((ldg, p), 7, dtype=np.int8, order="F")
    buf[:n] = codes
    return torch.from_numpy(buf.ravel(order="F")).to(torch.device("cuda", 0))


def _case(gpu_lib, n, p, ldg, seed, stream=None, bad=False, rtol=1e-12):
    import torch

    import sodabayes_gb300 as sg
    rng = np.random.default_rng(seed)
    codes = rng.integers(0, 3, size=(n, p)).astype(np.int8)
    codes[:, 11 % p] = 0                       # monomorphic column
    freq = codes.sum(axis=0) / (2.0 * n)
    ref_codes = codes
    if bad:                                    # out-of-range codes count as 1 (a missing call)
        codes = codes.copy()
        codes[3, 5] = -9
        codes[n - 1, p - 2] = 3
        ref_codes = codes.copy()
        ref_codes[3, 5] = 1
        ref_codes[n - 1, p - 2] = 1
    dev = torch.device("cuda", 0)
    codes_d = _device_codes(codes, ldg)
    freq_d = torch.from_numpy(freq).to(dev)
    pred_d = torch.empty(n, dtype=torch.float64, device=dev)
    for call, mu in enumerate((3.25, -1.5)):
        eff = rng.standard_normal(p) * 0.05
        eff[7 % p] = 0.0
        eff_d = torch.from_numpy(eff).to(dev)
        pred_d.fill_(np.nan)
        torch.cuda.synchronize()
        assert _call(gpu_lib, codes_d, ldg, freq_d, eff_d, pred_d, n, p, mu, stream) == 0, call
        if stream is not None:
            stream.synchronize()
        torch.cuda.synchronize()
        got = pred_d.cpu().numpy()
        want = sg.predict(codes=ref_codes, freq=freq, mu=mu, effects=eff)
        assert np.all(np.isfinite(got))
        assert np.allclose(got, want, rtol=rtol, atol=rtol * np.max(np.abs(want))), call


def test_noalloc_dgv_matches_predict(gpu_lib):
    _case(gpu_lib, 1237, 3001, 1237, 17)


def test_noalloc_padded_codes_on_a_caller_stream(gpu_lib):
    import torch
    st = torch.cuda.Stream()
    _case(gpu_lib, 1000, 777, 1000 + 48, 18, stream=st)


def test_noalloc_more_than_65536_individuals(gpu_lib):
    _case(gpu_lib, 70001, 300, 70001, 19)


def test_noalloc_codes_outside_0_to_2_count_as_one(gpu_lib):
    _case(gpu_lib, 500, 64, 512, 20, bad=True)


def test_noalloc_rejects_oversized_input(gpu_lib):
    """nind beyond SODAGPU_NOALLOC_SCRATCH is refused (valid small buffers: nothing may launch)."""
    import torch

    from sodabayes_gb300 import _abi
    dev = torch.device("cuda", 0)
    codes_d = torch.zeros(64, dtype=torch.int8, device=dev)
    vec = torch.zeros(64, dtype=torch.float64, device=dev)
    too_many = 2 * 1024 * 1024 + 1
    rc = gpu_lib.sodagpu_compute_dgv_noalloc(too_many, 1, C.c_void_p(codes_d.data_ptr()), too_many,
                                             C.c_void_p(vec.data_ptr()), 0.0, C.c_void_p(vec.data_ptr()),
                                             C.c_void_p(vec.data_ptr()), None)
    assert rc == _abi.E_ARG
    assert torch.all(vec == 0)
