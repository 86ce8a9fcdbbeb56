"""The regular (non-SODA, -SODAOff) sampler of the CPU oracle
(regular_bayes, models.f90:607-962): configuration, the residual identity,
the BayesA accumulator difference from soda_bayes, and agreement with the
SODA sampler at the Monte-Carlo level (the reference's examples 1 and 2 show
the same agreement: posterior mean 68.6537 vs 68.6552)."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, make_config, synth

N, P = 200, 400


@pytest.fixture(scope="module")
def data():
    return synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.5, ncausal=20, h2=0.5, mean=10.0, seed=5))


def _opts(method, soda, **kw):
    base = dict(method=method, pi=0.95, numit=1000, burnin=100, thin=1, blocksize=100, seed=31,
                scale_va=0.05, df_va=4.0, scale_ve=0.5, df_ve=4.0, soda=soda)
    if method in ("BayesR", "BayesRc"):
        base.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    base.update(kw)
    return JobOptions(**base)


def _run(oracle_mod, data, opts, iters):
    G, y, _ = data
    cfg = make_config(N, P, opts)
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    o.load_pheno(y)
    assert o.build_z() == 0
    o.init_chains()
    o.run(iters)
    return o


def test_sodaoff_config():
    cfg = make_config(N, P, _opts("BayesC", False))
    assert cfg.sampler == 1 and cfg.blocksize == P and cfg.nblocks == 1
    # blocksize <= 1 (setup_soda, soda.f90:418-421) switches SODA off as well
    cfg = make_config(N, P, _opts("BayesC", True, blocksize=0, nthreads=1))
    assert cfg.sampler == 1
    assert make_config(N, P, _opts("BayesC", True)).sampler == 0


@pytest.mark.parametrize("method", ["BayesA", "BayesB", "BayesC", "BayesR"])
def test_regular_residual_identity(oracle_mod, data, method):
    """yadj = y - mu - X g after several sweeps (compute_residuals,
    utilities.f90:609-614), every SNP single-site."""
    _, y, _ = data
    o = _run(oracle_mod, data, _opts(method, False), 7)
    st = o.state()
    X = o.x()
    assert np.max(np.abs(st["yadj"] - (y - st["mu"] - X @ st["g"]))) <= 1e-10 * np.max(np.abs(y))
    assert st["included"] == int(np.sum(st["cls"] > 1)) or method == "BayesA"


def test_regular_bayesa_keeps_no_varstore(oracle_mod, data):
    """regular_bayes accumulates varstore only for methods other than BayesA
    (models.f90:893-896); soda_bayes for every method (models.f90:530)."""
    reg = _run(oracle_mod, data, _opts("BayesA", False, burnin=2), 6).results()
    sod = _run(oracle_mod, data, _opts("BayesA", True, burnin=2), 6).results()
    assert np.all(reg["varstore"] == 0.0) and np.all(sod["varstore"] > 0.0)


def test_regular_and_soda_agree_in_posterior(oracle_mod, data):
    """Free-running BayesC chains of the two samplers: posterior-mean genomic
    values correlate to Monte-Carlo error."""
    res = {}
    for soda in (False, True):
        o = _run(oracle_mod, data, _opts("BayesC", soda), 1000)
        r = o.results()
        res[soda] = o.compute_dgv(r["mu_store"], r["gstore"])
    assert np.corrcoef(res[False], res[True])[0, 1] >= 0.98
