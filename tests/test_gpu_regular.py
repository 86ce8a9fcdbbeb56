"""The regular (non-SODA, -SODAOff) sampler on the GPU (one CTA per chain,
every SNP single-site in order, regular_bayes, models.f90:607-962) against
the CPU oracle fed the same counter-based draws.  FP64 throughout: class
indicators identical, effects, residuals and scalars within 1e-10 relative
after one iteration and 1e-9 after a dozen (the GPU's tree reductions round
differently from the oracle's sequential sums)."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu

N, P = 300, 700
GROUPS = (np.arange(P) % 3 + 1).astype(np.int32)


@pytest.fixture(scope="module")
def data():
    return synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.5, ncausal=25, h2=0.5, mean=30.0, seed=17))


def _opts(method, **kw):
    base = dict(method=method, pi=0.99, numit=100, burnin=3, thin=2, seed=555, scale_va=0.02, df_va=4.0,
                scale_ve=0.02, df_ve=4.0, precision="fp64", soda=False)
    if method in ("BayesR", "BayesRc"):
        base.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    if method == "BayesRc":
        base.update(ngroup=3)
    base.update(kw)
    return JobOptions(**base)


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


def _compare(job, o, tol, chain=0):
    sg, so = job.state(chain), o.state(chain)
    assert np.array_equal(sg["cls"], so["cls"])
    assert _rel(sg["g"], so["g"]) <= tol
    assert _rel(sg["yadj"], so["yadj"]) <= tol
    assert _rel(sg["vara_s"], so["vara_s"]) <= tol or np.all(so["vara_s"] == 0)
    for k in ("mu", "vare", "vara"):
        assert abs(sg[k] - so[k]) <= tol * max(1e-300, abs(so[k])), k
    assert sg["included"] == so["included"]


@pytest.mark.parametrize("method", ["BayesA", "BayesB", "BayesC", "BayesCpi", "BayesR", "BayesRc"])
def test_regular_chain_matches_oracle(gpu_lib, oracle_mod, data, method):
    G, y, _ = data
    cfg = make_config(N, P, _opts(method, chains=2))
    job, o = SodaJob(cfg), oracle_mod.Oracle(cfg)
    for s in (job, o):
        s.load_genotypes(G)
        s.load_pheno(y)
        if cfg.method == 6:
            s.set_groups(GROUPS)
    assert job.build_z() == 0 and o.build_z() == 0
    job.init_chains()
    o.init_chains()
    _compare(job, o, 1e-12)
    rows_g, rows_o = [], []
    job.run(1, trace=lambda r: rows_g.append((r.chain, r.rep, r.included, r.mu, r.vare, r.vara)))
    o.run(1, trace=lambda r: rows_o.append((r.chain, r.rep, r.included, r.mu, r.vare, r.vara)))
    for c in range(2):
        _compare(job, o, 1e-10, c)
    job.run(11, trace=lambda r: rows_g.append((r.chain, r.rep, r.included, r.mu, r.vare, r.vara)))
    o.run(11, trace=lambda r: rows_o.append((r.chain, r.rep, r.included, r.mu, r.vare, r.vara)))
    for c in range(2):
        _compare(job, o, 1e-9, c)
    assert len(rows_g) == len(rows_o) == 12
    for a, b in zip(sorted(rows_g), sorted(rows_o)):
        assert a[:3] == b[:3] and np.allclose(a[3:], b[3:], rtol=1e-9, atol=0)
    rg, ro = job.results(), o.results()
    assert _rel(rg["gstore"], ro["gstore"]) <= 1e-9
    assert np.array_equal(rg["indiststore"], ro["indiststore"])
    assert np.allclose(rg["varstore"], ro["varstore"], rtol=1e-9, atol=0)
    for k in ("mu_store", "vare_store", "vara_store", "included_store"):
        assert abs(rg[k] - ro[k]) <= 1e-9 * max(1e-300, abs(ro[k])), k
    job.close()
