"""Parity at the sizes of the benchmark configurations, GPU (C ABI) against
the CPU oracle fed the same counter-based draws.

Config 1 in full: SODA BayesC, FP64, one chain, n = 1,000, p = 5,000, subsets
of 500, pi fixed at 0.01 (the reference's -pi is the fraction of zero
effects, so -pi 0.99), genotypes Binomial(2, maf), maf ~ U(0.05, 0.5).
Config 2 in full: SODA BayesR (four classes 0, 1e-4, 1e-3, 1e-2), n = 5,000,
p = 50,000, subsets of 1,000, LD generator (50-SNP AR(1) blocks, rho 0.7).

Tolerances: FP64 — identical class indicators, effects / residuals / scalars
within 1e-10 relative after one iteration and 1e-9 after three (rounding of
the GPU's tree reductions compounds through the chain).  FP32 (config 2) —
at least 99% identical class indicators and effects within 1e-3 relative RMS
after one iteration."""
import os

import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


def _same(sg, so, tol):
    assert np.array_equal(sg["cls"], so["cls"])
    assert _rel(sg["g"], so["g"]) <= tol
    assert _rel(sg["yadj"], so["yadj"]) <= tol
    assert _rel(sg["yaadj"], so["yaadj"]) <= tol
    for k in ("mu", "vare", "vara"):
        assert abs(sg[k] - so[k]) <= tol * max(1e-300, abs(so[k])), k
    assert sg["included"] == so["included"]


def _pair(oracle_mod, G, y, opts):
    oracle_mod.set_threads(os.cpu_count() or 1)
    cfg = make_config(G.shape[0], G.shape[1], opts)
    job = SodaJob(cfg)
    job.load_genotypes(G)
    job.load_pheno(y)
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    o.load_pheno(y)
    assert job.build_z() == o.build_z()
    _, xd, _ = job.z()
    _, xo, _ = o.z()
    assert _rel(xd, xo) <= 1e-12
    job.init_chains()
    o.init_chains()
    return job, o


def test_config1_bayesc_fp64_against_oracle(gpu_lib, oracle_mod):
    spec = synth.CONFIGS["c1"]
    G, y, _ = synth.make(spec)
    opts = JobOptions(method="BayesC", pi=0.99, blocksize=500, numit=2000, burnin=500, seed=20260001,
                      precision="fp64", scale_va=1.0, df_va=4.0, scale_ve=float(np.var(y)) / 2, df_ve=4.0)
    job, o = _pair(oracle_mod, G, y, opts)
    try:
        assert job.cfg.nblocks == 10
        job.run(1)
        o.run(1)
        _same(job.state(), o.state(), 1e-10)
        job.run(2)
        o.run(2)
        _same(job.state(), o.state(), 1e-9)
    finally:
        job.close()
        o.close()


@pytest.fixture(scope="module")
def c2():
    spec = synth.CONFIGS["c2"]
    G, y, _ = synth.make(spec)
    return G, y


def _c2_opts(prec):
    return dict(method="BayesR", nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2), blocksize=1000, numit=5000, burnin=0,
                seed=20260002, precision=prec, scale_va=1.0, df_va=4.0, scale_ve=1.0, df_ve=4.0)


@pytest.fixture(scope="module")
def c2_oracle(gpu_lib, oracle_mod, c2):
    """Oracle states after one and three iterations of config 2 on the GPU's Z.  The sweep is compared
    on one Z: its factor has the smallest eigenvalue 0.001 (soda.f90:485), so the 1e-12 relative
    difference between the GPU's Lanczos d and the oracle's power-method d moves U by ~1e-9, which
    would reach the draws.  The Z build itself is compared with the oracle's at config 1."""
    G, y = c2
    cfg = make_config(G.shape[0], G.shape[1], JobOptions(**_c2_opts("fp64")))
    with SodaJob(cfg) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        assert job.build_z() == 0
        xa, xxd, _ = job.z()
    oracle_mod.set_threads(os.cpu_count() or 1)
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    o.load_pheno(y)
    o.set_z(xa, xxd)
    del xa
    o.init_chains()
    o.run(1)
    s1 = o.state()
    o.run(2)
    s3 = o.state()
    o.close()
    return {"xxd": xxd, 1: s1, 3: s3}


def test_config2_bayesr_fp64_against_oracle(gpu_lib, c2, c2_oracle):
    G, y = c2
    cfg = make_config(G.shape[0], G.shape[1], JobOptions(**_c2_opts("fp64")))
    with SodaJob(cfg) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        assert job.build_z() == 0
        assert np.array_equal(job.z()[1], c2_oracle["xxd"])   # the Z build is deterministic
        job.init_chains()
        job.run(1)
        _same(job.state(), c2_oracle[1], 1e-10)
        job.run(2)
        _same(job.state(), c2_oracle[3], 1e-9)


def test_config2_bayesr_fp32_against_oracle(gpu_lib, c2, c2_oracle):
    G, y = c2
    cfg = make_config(G.shape[0], G.shape[1], JobOptions(**_c2_opts("fp32")))
    with SodaJob(cfg) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        job.run(1)
        sg, so = job.state(), c2_oracle[1]
    agree = np.mean(sg["cls"] == so["cls"])
    rel = np.sqrt(np.mean((sg["g"] - so["g"]) ** 2)) / np.sqrt(np.mean(so["g"] ** 2))
    assert agree >= 0.99, agree
    assert rel <= 1e-3, rel
    assert abs(sg["vare"] / so["vare"] - 1.0) <= 1e-3
