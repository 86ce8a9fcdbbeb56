"""Argument checks of the batch entry points (sodagpu_batch_*), on the CPU:
they run before any CUDA call, so the library answers them without a GPU."""
import ctypes as C

from sodabayes_gb300 import _abi


def test_batch_entry_points_refuse_bad_arguments(gpu_lib):
    lib = gpu_lib
    out = C.c_void_p()
    jobs = (C.c_void_p * 2)(None, None)
    assert lib.sodagpu_batch_create(None, jobs, 2, 0) == -1   # SODAGPU_E_ARG
    assert lib.sodagpu_batch_create(C.byref(out), None, 2, 0) < 0
    assert lib.sodagpu_batch_create(C.byref(out), jobs, 0, 0) < 0
    assert lib.sodagpu_batch_create(C.byref(out), jobs, _abi.MAXJOBS + 1, 0) < 0
    assert lib.sodagpu_batch_create(C.byref(out), jobs, 2, 0) < 0          # null jobs
    assert lib.sodagpu_batch_create(C.byref(out), jobs, 2, 0x40) < 0       # unknown flag
    assert not out.value
    assert lib.sodagpu_batch_run(None, 1) < 0
    assert lib.sodagpu_batch_timings(None, None, None) < 0
    lib.sodagpu_batch_destroy(None)   # a no-op
    msg = lib.sodagpu_last_error().decode()
    assert msg
