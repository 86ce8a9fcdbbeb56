"""The C-ABI library loads and exports every entry point include/sodagpu.h
declares; host-side calls that need no GPU behave like the reference."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    hdr = open(os.path.join(ROOT, "include", "sodagpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(sodagpu_[a-z_0-9]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def lib():
    from sodabayes_gb300 import build as _b
    _b.build()
    import sodabayes_gb300
    return sodabayes_gb300.library()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version_and_errstr(lib):
    assert lib.sodagpu_abi_version() == 1
    assert lib.sodagpu_errstr(-5).decode().startswith("d*I - X'X")
    assert lib.sodagpu_errstr(0).decode() == "ok"


@pytest.mark.parametrize("nloci,nthreads,bsz,nbk,want", [
    (9346, 4, 0, 10, (935, 10, 9346 - 934 * 10, False)),    # example1: -nblocks 10
    (5000, 1, 500, 0, (500, 10, 10, False)),                # config 1: -blocksize 500
    (5001, 1, 500, 0, (500, 11, 11, False)),
    (100, 1, 0, 0, (1, 100, 100, True)),                    # blocksize = nthreads = 1 -> SODA off
    (100, 8, 0, 0, (8, 13, 13, False)),
])
def test_block_layout(lib, nloci, nthreads, bsz, nbk, want):
    """setup_soda block sizing (soda.f90:407-421), C ABI and Python restatement."""
    import sodabayes_gb300 as sg
    assert sg.block_layout(nloci, nthreads, bsz, nbk) == want
    assert sg.block_layout_py(nloci, nthreads, bsz, nbk) == want


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import sodabayes_gb300 as sg
    cfg = sg.make_config(10, 20, sg.JobOptions(method="BayesC", blocksize=5))
    ctx = C.c_void_p()
    rc = lib.sodagpu_create(C.byref(cfg), C.byref(ctx))
    assert rc == -7 and not ctx
    assert "device" in lib.sodagpu_last_error().decode()
