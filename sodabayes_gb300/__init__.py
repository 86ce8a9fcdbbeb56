"""sodabayes_gb300 — GB300-native SODA Gibbs sampler behind SODABayes' entry points.

The compute path is libsodagpu.so (CUDA, sm_103a; C ABI in include/sodagpu.h).
This module is the Python host mirror of the reference's option handling
(useroptions.f90) and of its job flow (SODABayes.f90:112-165) on top of that
ABI.  There is no CPU fallback: without the shared library, or without an
sm_103a GPU, every call raises SodaGpuError.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import (BAYES_A, BAYES_B, BAYES_C, BAYES_CPI, BAYES_R, BAYES_RC, FP8, FP32, FP64, GENO_BED,
                   GENO_CODES, GENO_DEVICE_PTR, METHODS, PRECISIONS, Config, TraceRow, fround)

__all__ = ["SodaGpuError", "JobOptions", "make_config", "block_layout", "SodaJob", "predict", "library",
           "METHODS", "PRECISIONS", "TraceRow"]

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libsodagpu.so")


class SodaGpuError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        self.code = code
        super().__init__(f"{where}: {msg or 'error'} (code {code})")


_lib: Optional[C.CDLL] = None


def library() -> C.CDLL:
    """Loads libsodagpu.so (built by sodabayes_gb300.build); raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SodaGpuError(-7, "library", f"{LIB_PATH} is missing; run `python -m sodabayes_gb300.build`")
        _lib = _abi.bind(C.CDLL(LIB_PATH), _abi.PROTOTYPES)
    return _lib


def _check(rc: int, where: str) -> None:
    if rc != 0:
        lib = library()
        msg = lib.sodagpu_last_error().decode(errors="replace")
        raise SodaGpuError(rc, where, msg or lib.sodagpu_errstr(rc).decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def block_layout(nloci: int, nthreads: int = 1, blocksize: int = 0, nblocks: int = 0):
    """setup_soda's block sizing (soda.f90:407-421): (blocksize, nblocks, blockt, soda_off)."""
    bs, nb, bt = C.c_int32(), C.c_int32(), C.c_int32()
    off = library().sodagpu_block_layout(nloci, nthreads, blocksize, nblocks, C.byref(bs), C.byref(nb), C.byref(bt))
    if off < 0:
        _check(off, "sodagpu_block_layout")
    return bs.value, nb.value, bt.value, bool(off == 1)


def block_layout_py(nloci: int, nthreads: int = 1, blocksize: int = 0, nblocks: int = 0):
    """Pure restatement of soda.f90:407-421 (no library needed)."""
    import math
    if blocksize > 0:
        bs = blocksize
        nb = math.ceil(nloci / bs)
        bt = nb
    elif nblocks > 0:
        nb = nblocks
        bs = math.ceil(nloci / nb)
        bt = nloci - (bs - 1) * nb
    else:
        bs = nthreads
        nb = math.ceil(nloci / max(bs, 1))
        bt = nb
    return bs, nb, bt, bs <= 1


@dataclass
class JobOptions:
    """The option table of useroptions.f90:23-55 that the SODA path reads, with
    the reference's defaults, plus the GPU knobs (precision, chains)."""
    method: str = "BayesCpi"
    pi: float = 0.99
    scale_va: float = 0.01
    scale_ve: float = 0.01
    df_va: float = 0.01
    df_ve: float = 0.01
    alpha: Sequence[float] = (1.0,)
    numit: int = 50000
    burnin: int = 5000
    thin: int = 1
    nmix: int = 2
    mix: Sequence[float] = (0.0, 1.0)
    seed: int = 0
    nthreads: int = 1
    blocksize: int = 0
    nblocks: int = 0
    ngroup: int = 1
    precision: str = "fp64"
    chains: int = 1
    recal_every: int = 1000
    vara0: float = 0.0
    kernels: str = "auto"          # "auto" (tensor cores where they apply) or "cuda_cores"
    soda: bool = True              # -SODAOn / -SODAOff: False runs the regular sampler (models.f90:607-962)


def make_config(nind: int, nloci: int, opts: JobOptions) -> Config:
    """Applies parse_method/parse_nmix/parse_pi/parse_priors/parse_soda
    (useroptions.f90:375-537) to `opts` and fills the C config struct."""
    names = {k.lower(): v for k, v in METHODS.items()}
    m = names.get(opts.method.lower())
    if m is None:
        raise ValueError("supported methods: BayesA, BayesB, BayesC, BayesCpi, BayesR, and BayesRc")
    cfg = Config()
    cfg.nind, cfg.nloci, cfg.method = nind, nloci, m
    # parse_nmix (useroptions.f90:375-400)
    if opts.nmix > _abi.MAXDIST:
        raise ValueError(f"nmix is too big. maximum allowed: {_abi.MAXDIST}")
    nmix = 1 if m == BAYES_A else (2 if m in (BAYES_B, BAYES_C, BAYES_CPI) else opts.nmix)
    cfg.nmix = nmix
    cfg.ngroup = opts.ngroup if m == BAYES_RC else 1
    # parse_pi (useroptions.f90:429-440): only BayesB/BayesC read -pi
    pz = fround(opts.pi)
    if m in (BAYES_B, BAYES_C) and not (0.0 < pz < 1.0):
        raise ValueError("pi must be a value between 0 and 1")
    cfg.pizero = pz
    cfg.scale_va, cfg.scale_ve = fround(opts.scale_va), fround(opts.scale_ve)
    cfg.df_va, cfg.df_ve = fround(opts.df_va), fround(opts.df_ve)
    # parse_priors: -mix and -alpha (useroptions.f90:501-535)
    for j in range(_abi.MAXDIST):
        cfg.mix[j] = 0.0
        cfg.alpha[j] = 0.0
    if m in (BAYES_C, BAYES_CPI):
        cfg.mix[0], cfg.mix[1] = 0.0, 1.0
    elif m in (BAYES_R, BAYES_RC):
        if len(opts.mix) != nmix:
            raise ValueError(f"Number of mixture classes {nmix} but {len(opts.mix)} effect sizes specified (mix)")
        for j, v in enumerate(opts.mix):
            cfg.mix[j] = fround(v)
    if m in (BAYES_CPI, BAYES_R, BAYES_RC):
        al = list(opts.alpha)
        if len(al) == 1:
            al = al * nmix
        elif len(al) != nmix:
            raise ValueError(f"Number of mixture classes {nmix} but {len(al)} prior values for Dirichlet specified")
        for j, v in enumerate(al):
            cfg.alpha[j] = fround(v)
    cfg.numit, cfg.burnin, cfg.thin, cfg.seed = opts.numit, opts.burnin, opts.thin, opts.seed
    bs, nb, bt, off = block_layout_py(nloci, opts.nthreads, opts.blocksize, opts.nblocks)
    if off or not opts.soda:
        # -SODAOff, or blocksize <= 1 (setup_soda switches SODA off, soda.f90:418-421): the
        # regular sampler, which has no subsets
        cfg.sampler = 1
        bs, nb, bt = nloci, 1, 1
    cfg.blocksize, cfg.nblocks, cfg.blockt = bs, nb, bt
    cfg.precision = PRECISIONS[opts.precision] if isinstance(opts.precision, str) else int(opts.precision)
    cfg.chains = opts.chains
    cfg.recal_every = opts.recal_every
    cfg.vara0 = opts.vara0
    kern = {"auto": 0, "cuda_cores": 1}
    if opts.kernels not in kern:
        raise ValueError("kernels must be 'auto' or 'cuda_cores'")
    cfg.kernels = kern[opts.kernels]
    return cfg


class SodaJob:
    """One SODA job on the GPU: the sequence setup_soda -> soda_bayes of
    SODABayes.f90:139-142 through the C ABI."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        self._lib = library()
        self._ctx = C.c_void_p()
        _check(self._lib.sodagpu_create(C.byref(cfg), C.byref(self._ctx)), "sodagpu_create")
        self.n, self.p, self.chains = cfg.nind, cfg.nloci, cfg.chains

    def close(self) -> None:
        if self._ctx:
            self._lib.sodagpu_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup -----------------------------------------------------------------
    def load_genotypes(self, codes=None, bed: Optional[np.ndarray] = None, device_ptr: Optional[int] = None,
                       host_ptr: Optional[int] = None, layout: int = GENO_CODES) -> None:
        """codes: int8 (nind, nloci) 0/1/2 (column-major is copied as-is);
        bed: uint8 PLINK payload without the magic header;
        device_ptr / host_ptr: an address holding `layout` data (e.g. pinned memory)."""
        if host_ptr is not None:
            _check(self._lib.sodagpu_load_genotypes(self._ctx, C.c_void_p(host_ptr), layout),
                   "sodagpu_load_genotypes")
            return
        if device_ptr is not None:
            _check(self._lib.sodagpu_load_genotypes(self._ctx, C.c_void_p(device_ptr), layout | GENO_DEVICE_PTR),
                   "sodagpu_load_genotypes")
            return
        if bed is not None:
            b = np.ascontiguousarray(bed, dtype=np.uint8)
            _check(self._lib.sodagpu_load_genotypes(self._ctx, b.ctypes.data_as(C.c_void_p), GENO_BED),
                   "sodagpu_load_genotypes")
            return
        g = np.asfortranarray(codes, dtype=np.int8)
        if g.shape != (self.n, self.p):
            raise ValueError(f"codes must be ({self.n}, {self.p}), got {g.shape}")
        _check(self._lib.sodagpu_load_genotypes(self._ctx, g.ctypes.data_as(C.c_void_p), GENO_CODES),
               "sodagpu_load_genotypes")

    def freq(self) -> np.ndarray:
        out = np.empty(self.p)
        _check(self._lib.sodagpu_get_freq(self._ctx, _dp(out)), "sodagpu_get_freq")
        return out

    def load_pheno(self, y) -> None:
        yy = np.ascontiguousarray(y, dtype=np.float64)
        _check(self._lib.sodagpu_load_pheno(self._ctx, _dp(yy)), "sodagpu_load_pheno")

    def set_groups(self, groups) -> None:
        gg = np.ascontiguousarray(groups, dtype=np.int32)
        _check(self._lib.sodagpu_set_groups(self._ctx, _ip(gg)), "sodagpu_set_groups")

    def set_d_offset(self, delta: float) -> None:
        _check(self._lib.sodagpu_set_d_offset(self._ctx, float(delta)), "sodagpu_set_d_offset")

    def build_z(self, permvec=None) -> int:
        nsk = C.c_int32()
        pv = None if permvec is None else np.ascontiguousarray(permvec, dtype=np.int32)
        _check(self._lib.sodagpu_build_z(self._ctx, None if pv is None else _ip(pv), C.byref(nsk)),
               "sodagpu_build_z")
        return nsk.value

    def set_tape(self, tape) -> None:
        """Injected draws: every draw site of chain 0 takes its uniforms from
        `tape` (layout of sodagpu_set_tape); None removes it.  Call before
        init_chains."""
        if tape is None:
            _check(self._lib.sodagpu_set_tape(self._ctx, None, 0), "sodagpu_set_tape")
            return
        t = np.ascontiguousarray(tape, dtype=np.float64)
        _check(self._lib.sodagpu_set_tape(self._ctx, _dp(t), t.size), "sodagpu_set_tape")

    def init_chains(self) -> None:
        _check(self._lib.sodagpu_init_chains(self._ctx), "sodagpu_init_chains")

    # -- sampling --------------------------------------------------------------
    def run(self, iters: int, trace: Optional[Callable[[TraceRow], None]] = None) -> None:
        if trace is None:
            cb = _abi.TRACE_CB()
        else:
            cb = _abi.TRACE_CB(lambda user, row: trace(row.contents))
        _check(self._lib.sodagpu_run(self._ctx, int(iters), cb, None), "sodagpu_run")

    def state(self, chain: int = 0) -> dict:
        g = np.empty(self.p)
        cls = np.empty(self.p, dtype=np.int32)
        vs = np.empty(self.p)
        r = np.empty(self.n)
        ra = np.empty(self.cfg.blocksize)
        sc = np.empty(4)
        _check(self._lib.sodagpu_get_state(self._ctx, chain, _dp(g), _ip(cls), _dp(vs), _dp(r), _dp(ra), _dp(sc)),
               "sodagpu_get_state")
        return {"g": g, "cls": cls, "vara_s": vs, "yadj": r, "yaadj": ra, "mu": sc[0], "vare": sc[1],
                "vara": sc[2], "included": int(sc[3])}

    def set_state(self, chain: int, g, cls, vara_s, yadj, yaadj, mu: float, vare: float, vara: float,
                  included: int = 0, pi=None) -> None:
        """Loads one chain's state (the inverse of state()); pi is the
        (ngroup, nmix) table of mixture proportions, or None to keep it."""
        gg = np.ascontiguousarray(g, dtype=np.float64)
        cc = np.ascontiguousarray(cls, dtype=np.int32)
        vv = np.ascontiguousarray(vara_s, dtype=np.float64)
        rr = np.ascontiguousarray(yadj, dtype=np.float64)
        ra = np.zeros(self.cfg.blocksize)
        ra[:min(len(yaadj), len(ra))] = np.asarray(yaadj, dtype=np.float64)[:len(ra)]
        sc = np.array([mu, vare, vara, included], dtype=np.float64)
        pp = None if pi is None else np.asfortranarray(pi, dtype=np.float64)
        if gg.shape != (self.p,) or cc.shape != (self.p,) or vv.shape != (self.p,) or rr.shape != (self.n,):
            raise ValueError("g, cls, vara_s must have nloci entries and yadj nind")
        _check(self._lib.sodagpu_set_state(self._ctx, chain, _dp(gg), _ip(cc), _dp(vv), _dp(rr), _dp(ra), _dp(sc),
                                           None if pp is None else pp.ctypes.data_as(C.POINTER(C.c_double))),
               "sodagpu_set_state")

    def set_iteration(self, rep: int) -> None:
        _check(self._lib.sodagpu_set_iteration(self._ctx, int(rep)), "sodagpu_set_iteration")

    def subset_rhs(self, b: int) -> np.ndarray:
        """(chains, N_b) conditional right-hand sides of subset b on the current state."""
        ls, le = self.subset_bounds(b)
        nsnp = le - ls
        out = np.empty(self.chains * nsnp)
        _check(self._lib.sodagpu_subset_rhs(self._ctx, int(b), _dp(out)), "sodagpu_subset_rhs")
        return out.reshape(self.chains, nsnp)

    def subset_bounds(self, b: int):
        """0-based [first, end) subset positions of subset b (models.f90:136-142)."""
        bs, bt, p = self.cfg.blocksize, self.cfg.blockt, self.p
        blocki = b + 1
        if blocki <= bt:
            ls = (blocki - 1) * bs + 1
            le = min(ls + bs - 1, p)
        else:
            ls = bs * bt + (blocki - bt - 1) * (bs - 1) + 1
            le = min(ls + bs - 2, p)
        return ls - 1, le

    def run_subset(self, b: int) -> None:
        _check(self._lib.sodagpu_run_subset(self._ctx, int(b)), "sodagpu_run_subset")

    def results(self, chain: int = 0) -> dict:
        p, nm, ng = self.p, self.cfg.nmix, self.cfg.ngroup
        gs = np.empty(p)
        ind = np.empty((p, nm), order="F")
        vss = np.empty(p)
        sc = np.empty(4)
        snp = np.empty((ng, nm), order="F")
        pst = np.empty((ng, nm), order="F")
        var = np.empty((ng, nm), order="F")
        _check(self._lib.sodagpu_get_results(self._ctx, chain, _dp(gs), ind.ctypes.data_as(C.POINTER(C.c_double)),
                                             _dp(vss), _dp(sc), snp.ctypes.data_as(C.POINTER(C.c_double)),
                                             pst.ctypes.data_as(C.POINTER(C.c_double)),
                                             var.ctypes.data_as(C.POINTER(C.c_double))), "sodagpu_get_results")
        return {"gstore": gs, "indiststore": ind, "vara_sstore": vss, "mu_store": sc[0], "vare_store": sc[1],
                "vara_store": sc[2], "included_store": sc[3], "snpstore": snp, "pstore": pst, "varstore": var}

    def z(self):
        xa = np.empty((self.cfg.blocksize, self.p), order="F")
        xxd = np.empty(self.cfg.nblocks)
        skip = np.empty(self.p, dtype=np.int32)
        _check(self._lib.sodagpu_get_z(self._ctx, xa.ctypes.data_as(C.POINTER(C.c_double)), _dp(xxd), _ip(skip)),
               "sodagpu_get_z")
        return xa, xxd, skip

    def compute_dgv(self, mu: float, effects) -> np.ndarray:
        e = np.ascontiguousarray(effects, dtype=np.float64)
        out = np.empty(self.n)
        _check(self._lib.sodagpu_compute_dgv(self._ctx, float(mu), _dp(e), _dp(out)), "sodagpu_compute_dgv")
        return out

    def timings(self):
        """(build_z seconds, last run seconds, last run device milliseconds)"""
        b, r, d = C.c_double(), C.c_double(), C.c_double()
        _check(self._lib.sodagpu_timings(self._ctx, C.byref(b), C.byref(r), C.byref(d)), "sodagpu_timings")
        return b.value, r.value, d.value

    def profile_kernels(self, iters: int) -> dict:
        """Per-kernel-class device time (ms) and launch counts over `iters` eager iterations."""
        names = ("rhs", "update", "mu", "other", "draw")
        ms = np.zeros(len(names))
        n = np.zeros(len(names), dtype=np.int32)
        _check(self._lib.sodagpu_profile_kernels(self._ctx, int(iters), _dp(ms), _ip(n)), "sodagpu_profile_kernels")
        return {names[k]: (float(ms[k]), int(n[k])) for k in range(len(names))}


class SodaBatch:
    """Several SodaJob analyses run together: every kernel of an iteration is
    launched once over all of them (sodagpu_batch_create).  Each job keeps
    its own results, exactly those it would give on its own; read them with
    the job's methods after run()."""

    def __init__(self, jobs, solo_splits: bool = False):
        self._lib = library()
        self.jobs = list(jobs)
        arr = (C.c_void_p * len(self.jobs))(*[j._ctx.value for j in self.jobs])
        self._b = C.c_void_p()
        flags = _abi.BATCH_SOLO_SPLITS if solo_splits else 0
        _check(self._lib.sodagpu_batch_create(C.byref(self._b), arr, len(self.jobs), flags), "sodagpu_batch_create")

    def run(self, iters: int) -> None:
        _check(self._lib.sodagpu_batch_run(self._b, int(iters)), "sodagpu_batch_run")

    def timings(self):
        """(device milliseconds of the last run, subset steps per iteration)"""
        ms, st = C.c_double(), C.c_int32()
        _check(self._lib.sodagpu_batch_timings(self._b, C.byref(ms), C.byref(st)), "sodagpu_batch_timings")
        return ms.value, st.value

    def close(self) -> None:
        if self._b:
            self._lib.sodagpu_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def autotune_batch(n, p, iters: int, max_blocksize: int = 2000, model=None):
    """Subset sizes for a batch (sodagpu_autotune_batch): returns (blocksizes,
    steps, modelled seconds)."""
    lib = library()
    nn = np.ascontiguousarray(n, dtype=np.int32)
    pp = np.ascontiguousarray(p, dtype=np.int32)
    bs = np.zeros(nn.shape[0], dtype=np.int32)
    steps, secs = C.c_int32(), C.c_double()
    m = None if model is None else np.ascontiguousarray(model, dtype=np.float64)
    _check(lib.sodagpu_autotune_batch(nn.shape[0], _ip(nn), _ip(pp), int(iters), int(max_blocksize),
                                      None if m is None else _dp(m), _ip(bs), C.byref(steps), C.byref(secs)),
           "sodagpu_autotune_batch")
    return bs, steps.value, secs.value


def predict(codes=None, freq=None, mu: float = 0.0, effects=None, bed: Optional[np.ndarray] = None,
            nind: Optional[int] = None) -> np.ndarray:
    """Prediction mode (utilities.f90:540-553, 616-622): mu + X*effects with
    the centring of an external .frq file."""
    lib = library()
    fr = np.ascontiguousarray(freq, dtype=np.float64)
    e = np.ascontiguousarray(effects, dtype=np.float64)
    p = fr.shape[0]
    if bed is not None:
        n = int(nind)
        buf = np.ascontiguousarray(bed, dtype=np.uint8)
        layout = GENO_BED
    else:
        g = np.asfortranarray(codes, dtype=np.int8)
        n = g.shape[0]
        buf = g
        layout = GENO_CODES
    out = np.empty(n)
    _check(lib.sodagpu_predict(n, p, buf.ctypes.data_as(C.c_void_p), layout, _dp(fr), float(mu), _dp(e), _dp(out)),
           "sodagpu_predict")
    return out
