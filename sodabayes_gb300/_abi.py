"""ctypes mirror of include/sodagpu.h (structs, enums, prototypes)."""
from __future__ import annotations

import ctypes as C

MAXDIST = 20
MAXGRP = 100
TAPE_W = 32          # uniforms per draw site of an injected-draw tape

BAYES_A, BAYES_B, BAYES_C, BAYES_CPI, BAYES_R, BAYES_RC = 1, 2, 3, 4, 5, 6
METHODS = {"BayesA": BAYES_A, "BayesB": BAYES_B, "BayesC": BAYES_C, "BayesCpi": BAYES_CPI,
           "BayesR": BAYES_R, "BayesRc": BAYES_RC}
FP64, FP32, FP8 = 0, 1, 2
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp8": FP8}
GENO_CODES, GENO_BED, GENO_DEVICE_PTR = 0, 1, 0x100

E_ARG, E_STATE, E_NOMEM, E_CUDA, E_NOTPSD, E_TIMEOUT, E_NODEVICE, E_UNSUPPORTED = -1, -2, -3, -4, -5, -6, -7, -8


class Config(C.Structure):
    _fields_ = [
        ("nind", C.c_int32), ("nloci", C.c_int32), ("method", C.c_int32), ("nmix", C.c_int32),
        ("ngroup", C.c_int32), ("blocksize", C.c_int32), ("nblocks", C.c_int32), ("blockt", C.c_int32),
        ("numit", C.c_int32), ("burnin", C.c_int32), ("thin", C.c_int32), ("precision", C.c_int32),
        ("chains", C.c_int32), ("recal_every", C.c_int32), ("seed", C.c_int64),
        ("pizero", C.c_double), ("scale_va", C.c_double), ("scale_ve", C.c_double),
        ("df_va", C.c_double), ("df_ve", C.c_double),
        ("mix", C.c_double * MAXDIST), ("alpha", C.c_double * MAXDIST), ("vara0", C.c_double),
        ("kernels", C.c_int32), ("sampler", C.c_int32), ("reserved", C.c_int32 * 6),
    ]


class TraceRow(C.Structure):
    _fields_ = [
        ("chain", C.c_int32), ("rep", C.c_int32), ("included", C.c_int32), ("pad", C.c_int32),
        ("mu", C.c_double), ("vare", C.c_double), ("vara", C.c_double),
        ("snpindist", C.c_int32 * MAXDIST), ("varindist", C.c_double * MAXDIST),
    ]


TRACE_CB = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(TraceRow))

_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)

# name -> (restype, argtypes); every function returns an int status unless noted
PROTOTYPES = {
    "sodagpu_abi_version": (C.c_int, []),
    "sodagpu_errstr": (C.c_char_p, [C.c_int]),
    "sodagpu_last_error": (C.c_char_p, []),
    "sodagpu_block_layout": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _IP, _IP, _IP]),
    "sodagpu_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "sodagpu_load_genotypes": (C.c_int, [_P, _P, C.c_int32]),
    "sodagpu_get_freq": (C.c_int, [_P, _DP]),
    "sodagpu_load_pheno": (C.c_int, [_P, _DP]),
    "sodagpu_set_groups": (C.c_int, [_P, _IP]),
    "sodagpu_build_z": (C.c_int, [_P, _IP, _IP]),
    "sodagpu_set_d_offset": (C.c_int, [_P, C.c_double]),
    "sodagpu_set_tape": (C.c_int, [_P, _DP, C.c_size_t]),
    "sodagpu_init_chains": (C.c_int, [_P]),
    "sodagpu_run": (C.c_int, [_P, C.c_int32, TRACE_CB, _P]),
    "sodagpu_get_results": (C.c_int, [_P, C.c_int32, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
    "sodagpu_get_state": (C.c_int, [_P, C.c_int32, _DP, _IP, _DP, _DP, _DP, _DP]),
    "sodagpu_set_state": (C.c_int, [_P, C.c_int32, _DP, _IP, _DP, _DP, _DP, _DP, _DP]),
    "sodagpu_set_iteration": (C.c_int, [_P, C.c_int32]),
    "sodagpu_subset_rhs": (C.c_int, [_P, C.c_int32, _DP]),
    "sodagpu_run_subset": (C.c_int, [_P, C.c_int32]),
    "sodagpu_get_z": (C.c_int, [_P, _DP, _DP, _IP]),
    "sodagpu_compute_dgv": (C.c_int, [_P, C.c_double, _DP, _DP]),
    "sodagpu_predict": (C.c_int, [C.c_int32, C.c_int32, _P, C.c_int32, _DP, C.c_double, _DP, _DP]),
    "sodagpu_timings": (C.c_int, [_P, _DP, _DP, _DP]),
    "sodagpu_profile_kernels": (C.c_int, [_P, C.c_int32, _DP, _IP]),
    "sodagpu_compute_dgv_noalloc": (C.c_int, [C.c_int32, C.c_int32, _P, C.c_int32, _P, C.c_double, _P, _P, _P]),
    "sodagpu_batch_create": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.c_int32, C.c_int32]),
    "sodagpu_batch_run": (C.c_int, [_P, C.c_int32]),
    "sodagpu_batch_timings": (C.c_int, [_P, _DP, _IP]),
    "sodagpu_batch_destroy": (None, [_P]),
    "sodagpu_autotune_batch": (C.c_int, [C.c_int32, _IP, _IP, C.c_int32, C.c_int32, _DP, _IP, _IP, _DP]),
    "sodagpu_destroy": (None, [_P]),
}

MAXJOBS = 64
BATCH_SOLO_SPLITS = 1


def bind(lib: C.CDLL, prototypes: dict) -> C.CDLL:
    for name, (res, args) in prototypes.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def fround(x: float) -> float:
    """Round a value through IEEE single precision, as the reference's
    cast_float() does for every REAL option (utilities.f90:168-171)."""
    import struct
    return struct.unpack("f", struct.pack("f", float(x)))[0]
