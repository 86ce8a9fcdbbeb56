"""ctypes binding of the CPU oracle (oracle/soda_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py.  Parity status: the prediction path is pinned
by the reference's shipped outputs; the Gibbs sweep and the Z build are a
restatement whose parity with reference runs is unpinned (no Fortran
compiler here, and the reference ships no tests).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from sodabayes_gb300 import _abi  # noqa: E402  (config struct shared with the C ABI)
from sodabayes_gb300._abi import TRACE_CB, Config  # noqa: E402

RNG_COUNTER, RNG_REFERENCE = 0, 1

_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
PROTOTYPES = {
    "oracle_create": (C.c_int, [C.POINTER(Config), C.c_int32, C.c_int32, C.POINTER(_P)]),
    "oracle_destroy": (None, [_P]),
    "oracle_set_omp_threads": (C.c_int, [C.c_int32]),
    "oracle_decode_bed": (C.c_int, [C.c_int32, C.c_int32, _P, _P]),
    "oracle_load_genotypes": (C.c_int, [_P, _P]),
    "oracle_get_freq": (C.c_int, [_P, _DP]),
    "oracle_get_x": (C.c_int, [_P, _DP]),
    "oracle_load_pheno": (C.c_int, [_P, _DP]),
    "oracle_set_groups": (C.c_int, [_P, _IP]),
    "oracle_permutate": (C.c_int, [_P, _IP]),
    "oracle_gram": (C.c_int, [_P, _IP, C.c_int32, _DP]),
    "oracle_build_z": (C.c_int, [_P, _IP, C.c_int64, C.c_double, _IP]),
    "oracle_get_z": (C.c_int, [_P, _DP, _DP, _IP]),
    "oracle_set_z": (C.c_int, [_P, _DP, _DP]),
    "oracle_set_tape": (C.c_int, [_P, _DP, C.c_int32, C.c_int32]),
    "oracle_tape_sites": (C.c_int, [_P]),
    "oracle_init_chains": (C.c_int, [_P]),
    "oracle_run": (C.c_int, [_P, C.c_int32, TRACE_CB, _P]),
    "oracle_run_blocks": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "oracle_set_sparse_state": (C.c_int, [_P, C.c_double, C.c_int64]),
    "oracle_get_state": (C.c_int, [_P, C.c_int32, _DP, _IP, _DP, _DP, _DP, _DP]),
    "oracle_get_results": (C.c_int, [_P, C.c_int32, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
    "oracle_compute_dgv": (C.c_int, [_P, C.c_double, _DP, _DP]),
    "oracle_predict": (C.c_int, [C.c_int32, C.c_int32, _P, _DP, C.c_double, _DP, _DP]),
    "oracle_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "oracle_ref_uniforms": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, _DP]),
    "oracle_counter_uniforms": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _DP]),
    "oracle_sample": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_int32, C.c_double, C.c_double, _DP]),
    "oracle_cholesky_pd": (C.c_int, [C.c_int32, _DP, _DP]),
    "oracle_cholesky_psd": (C.c_int, [C.c_int32, _DP, _IP, _IP]),
    "oracle_power_method": (C.c_int, [C.c_int32, _DP, _DP, C.c_int64, _DP, C.POINTER(C.c_int64)]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _build  # type: ignore
        path = _build.build()
        _lib = _abi.bind(C.CDLL(path), PROTOTYPES)
    return _lib


def _dp(a):
    return a.ctypes.data_as(_DP)


def _ip(a):
    return a.ctypes.data_as(_IP)


def _chk(rc, where):
    if rc != 0:
        raise RuntimeError(f"{where} failed with code {rc}")


def set_threads(n: int) -> int:
    return lib().oracle_set_omp_threads(n)


class Oracle:
    """CPU FP64 SODA job with the same entry points as sodabayes_gb300.SodaJob."""

    def __init__(self, cfg: Config, rng_mode: int = RNG_COUNTER, ref_threads: int = 1):
        self.cfg = cfg
        self.n, self.p = cfg.nind, cfg.nloci
        self._lib = lib()
        self._o = C.c_void_p()
        _chk(self._lib.oracle_create(C.byref(cfg), rng_mode, ref_threads, C.byref(self._o)), "oracle_create")

    def close(self):
        if self._o:
            self._lib.oracle_destroy(self._o)
            self._o = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_genotypes(self, codes):
        g = np.asfortranarray(codes, dtype=np.int8)
        _chk(self._lib.oracle_load_genotypes(self._o, g.ctypes.data_as(C.c_void_p)), "oracle_load_genotypes")

    def freq(self):
        out = np.empty(self.p)
        _chk(self._lib.oracle_get_freq(self._o, _dp(out)), "oracle_get_freq")
        return out

    def x(self):
        out = np.empty((self.n, self.p), order="F")
        _chk(self._lib.oracle_get_x(self._o, out.ctypes.data_as(_DP)), "oracle_get_x")
        return out

    def load_pheno(self, y):
        yy = np.ascontiguousarray(y, dtype=np.float64)
        _chk(self._lib.oracle_load_pheno(self._o, _dp(yy)), "oracle_load_pheno")

    def set_groups(self, groups):
        gg = np.ascontiguousarray(groups, dtype=np.int32)
        _chk(self._lib.oracle_set_groups(self._o, _ip(gg)), "oracle_set_groups")

    def permutate(self):
        out = np.empty(self.p, dtype=np.int32)
        _chk(self._lib.oracle_permutate(self._o, _ip(out)), "oracle_permutate")
        return out

    def gram(self, cols):
        cc = np.ascontiguousarray(cols, dtype=np.int32)
        A = np.empty((len(cc), len(cc)), order="F")
        _chk(self._lib.oracle_gram(self._o, _ip(cc), len(cc), A.ctypes.data_as(_DP)), "oracle_gram")
        return A

    def build_z(self, permvec=None, power_maxit: int = 0, d_offset: float = 0.0) -> int:
        nsk = C.c_int32()
        pv = None if permvec is None else np.ascontiguousarray(permvec, dtype=np.int32)
        rc = self._lib.oracle_build_z(self._o, None if pv is None else _ip(pv), power_maxit, d_offset, C.byref(nsk))
        _chk(rc, "oracle_build_z")
        return nsk.value

    def record_tape(self, reps: int) -> np.ndarray:
        """Records the uniforms of every draw site of iterations 0 .. reps-1
        into a new tape (reps x sites x TAPE_W), filled as the chain runs."""
        sites = self._lib.oracle_tape_sites(self._o)
        self._tape = np.zeros(reps * sites * _abi.TAPE_W)
        _chk(self._lib.oracle_set_tape(self._o, _dp(self._tape), reps, 1), "oracle_set_tape")
        return self._tape

    def play_tape(self, tape) -> None:
        """Draw sites take their uniforms from `tape` instead of the RNG."""
        sites = self._lib.oracle_tape_sites(self._o)
        self._tape = np.ascontiguousarray(tape, dtype=np.float64)
        reps = len(self._tape) // (sites * _abi.TAPE_W)
        _chk(self._lib.oracle_set_tape(self._o, _dp(self._tape), reps, 0), "oracle_set_tape")

    def set_z(self, xa, xxd):
        """Uses the given Z (identity order, no skipped SNPs) instead of building it."""
        a = np.asfortranarray(xa, dtype=np.float64)
        d = np.ascontiguousarray(xxd, dtype=np.float64)
        _chk(self._lib.oracle_set_z(self._o, a.ctypes.data_as(_DP), _dp(d)), "oracle_set_z")

    def z(self):
        xa = np.empty((self.cfg.blocksize, self.p), order="F")
        xxd = np.empty(self.cfg.nblocks)
        skip = np.empty(self.p, dtype=np.int32)
        _chk(self._lib.oracle_get_z(self._o, xa.ctypes.data_as(_DP), _dp(xxd), _ip(skip)), "oracle_get_z")
        return xa, xxd, skip

    def init_chains(self):
        _chk(self._lib.oracle_init_chains(self._o), "oracle_init_chains")

    def run(self, iters: int, trace=None):
        cb = TRACE_CB() if trace is None else TRACE_CB(lambda u, row: trace(row.contents))
        _chk(self._lib.oracle_run(self._o, int(iters), cb, None), "oracle_run")

    def run_blocks(self, first_block: int, nblocks_run: int, reps: int = 1):
        _chk(self._lib.oracle_run_blocks(self._o, first_block, nblocks_run, reps), "oracle_run_blocks")

    def set_sparse_state(self, incl: float, seed: int = 1):
        _chk(self._lib.oracle_set_sparse_state(self._o, float(incl), seed), "oracle_set_sparse_state")

    def state(self, chain: int = 0) -> dict:
        g = np.empty(self.p)
        cls = np.empty(self.p, dtype=np.int32)
        vs = np.empty(self.p)
        r = np.empty(self.n)
        ra = np.empty(self.cfg.blocksize)
        sc = np.empty(4)
        _chk(self._lib.oracle_get_state(self._o, chain, _dp(g), _ip(cls), _dp(vs), _dp(r), _dp(ra), _dp(sc)),
             "oracle_get_state")
        return {"g": g, "cls": cls, "vara_s": vs, "yadj": r, "yaadj": ra, "mu": sc[0], "vare": sc[1],
                "vara": sc[2], "included": int(sc[3])}

    def results(self, chain: int = 0) -> dict:
        p, nm, ng = self.p, self.cfg.nmix, self.cfg.ngroup
        gs = np.empty(p)
        ind = np.empty((p, nm), order="F")
        vss = np.empty(p)
        sc = np.empty(4)
        snp = np.empty((ng, nm), order="F")
        pst = np.empty((ng, nm), order="F")
        var = np.empty((ng, nm), order="F")
        _chk(self._lib.oracle_get_results(self._o, chain, _dp(gs), ind.ctypes.data_as(_DP), _dp(vss), _dp(sc),
                                          snp.ctypes.data_as(_DP), pst.ctypes.data_as(_DP),
                                          var.ctypes.data_as(_DP)), "oracle_get_results")
        return {"gstore": gs, "indiststore": ind, "vara_sstore": vss, "mu_store": sc[0], "vare_store": sc[1],
                "vara_store": sc[2], "included_store": sc[3], "snpstore": snp, "pstore": pst, "varstore": var}

    def compute_dgv(self, mu, effects):
        e = np.ascontiguousarray(effects, dtype=np.float64)
        out = np.empty(self.n)
        _chk(self._lib.oracle_compute_dgv(self._o, float(mu), _dp(e), _dp(out)), "oracle_compute_dgv")
        return out


def decode_bed(payload: np.ndarray, nind: int, nloci: int) -> np.ndarray:
    codes = np.empty((nind, nloci), dtype=np.int8, order="F")
    b = np.ascontiguousarray(payload, dtype=np.uint8)
    _chk(lib().oracle_decode_bed(nind, nloci, b.ctypes.data_as(C.c_void_p), codes.ctypes.data_as(C.c_void_p)),
         "oracle_decode_bed")
    return codes


def predict(codes, freq, mu, effects):
    g = np.asfortranarray(codes, dtype=np.int8)
    fr = np.ascontiguousarray(freq, dtype=np.float64)
    e = np.ascontiguousarray(effects, dtype=np.float64)
    out = np.empty(g.shape[0])
    _chk(lib().oracle_predict(g.shape[0], g.shape[1], g.ctypes.data_as(C.c_void_p), _dp(fr), float(mu), _dp(e),
                              _dp(out)), "oracle_predict")
    return out


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return list(o)


def ref_uniforms(seed, stream, count):
    out = np.empty(count)
    _chk(lib().oracle_ref_uniforms(seed, stream, count, _dp(out)), "oracle_ref_uniforms")
    return out


def counter_uniforms(seed, chain, it, slot, purpose, count):
    out = np.empty(count)
    _chk(lib().oracle_counter_uniforms(seed, chain, it, slot, purpose, count, _dp(out)), "oracle_counter_uniforms")
    return out


def sample(dist, mode, seed, count, a=0.0, b=1.0):
    k = int(a) if dist == 4 else 1
    out = np.empty(count * k)
    _chk(lib().oracle_sample(dist, mode, seed, count, a, b, _dp(out)), "oracle_sample")
    return out.reshape(count, k) if dist == 4 else out


def cholesky_pd(A):
    A = np.asfortranarray(A, dtype=np.float64)
    U = np.empty_like(A, order="F")
    st = lib().oracle_cholesky_pd(A.shape[0], A.ctypes.data_as(_DP), U.ctypes.data_as(_DP))
    return U, st


def cholesky_psd(A):
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    piv = np.empty(A.shape[0], dtype=np.int32)
    rank = C.c_int32()
    st = lib().oracle_cholesky_psd(A.shape[0], A.ctypes.data_as(_DP), _ip(piv), C.byref(rank))
    return A, piv, rank.value, st


def power_method(A, start, maxit):
    A = np.asfortranarray(A, dtype=np.float64)
    s = np.ascontiguousarray(start, dtype=np.float64)
    lam = C.c_double()
    its = C.c_int64()
    _chk(lib().oracle_power_method(A.shape[0], A.ctypes.data_as(_DP), _dp(s), maxit, C.byref(lam), C.byref(its)),
         "oracle_power_method")
    return lam.value, its.value
