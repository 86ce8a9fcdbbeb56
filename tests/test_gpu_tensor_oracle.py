"""The tensor-core sweep of the FP8 mode (k_rhs_tc, k_draw<FP8,C,TC>,
k_update_tc with 4 chains) against the FP64 CPU oracle fed the same
counter-based draws.

After one iteration each chain must agree with the oracle's on >= 99% of its
class indicators, with effects and residuals within 1e-3 relative RMS (the
bound of the reduced-precision modes against FP64).  The oracle restates the
reference's sweep in FP64; both build the same Z (checked to 1e-12 in d)."""
import os

import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu

N, P, S, C = 1000, 1700, 300, 4


@pytest.fixture(scope="module")
def data():
    return synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.6, ncausal=40, h2=0.5, mean=10.0, seed=35))


def _rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(1e-300, np.sqrt(np.mean(b ** 2))))


@pytest.mark.parametrize("method", ["BayesCpi", "BayesR"])
def test_tensor_core_sweep_against_oracle(gpu_lib, oracle_mod, data, method):
    G, y, _ = data
    kw = dict(method=method, pi=0.95, numit=100, burnin=2, thin=1, blocksize=S, seed=5151, chains=C,
              scale_va=0.05, df_va=4.0, scale_ve=0.5, df_ve=4.0)
    if method == "BayesR":
        kw.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    oracle_mod.set_threads(os.cpu_count() or 1)
    job = SodaJob(make_config(N, P, JobOptions(precision="fp8", **kw)))
    o = oracle_mod.Oracle(make_config(N, P, JobOptions(precision="fp64", **kw)))
    try:
        for side in (job, o):
            side.load_genotypes(G)
            side.load_pheno(y)
        assert job.build_z() == o.build_z()
        _, dg, _ = job.z()
        _, do, _ = o.z()
        assert np.max(np.abs(dg - do) / np.abs(do)) <= 1e-12
        job.init_chains()
        o.init_chains()
        o.run(1)
        job.run(1)
        for c in range(C):
            sg, so = job.state(c), o.state(c)
            agree = float(np.mean(sg["cls"] == so["cls"]))
            assert agree >= 0.99, (c, agree)
            assert _rel_rms(sg["g"], so["g"]) <= 1e-3, c
            assert _rel_rms(sg["yadj"], so["yadj"]) <= 1e-3, c
            assert abs(sg["vare"] - so["vare"]) <= 1e-3 * abs(so["vare"]), c
    finally:
        job.close()
        o.close()
