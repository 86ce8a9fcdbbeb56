"""One subset on one loaded state: the FP8 tensor-core path (16 chains,
k_rhs_tc / k_draw / k_update_tc) against the FP64 path, at the subset shapes
of config 3 (BayesCpi, n = 20,000, subsets of 2,000) and config 5 (BayesRc in
three annotation groups, four classes, n = 50,000, subsets of 1,000).

Both contexts load the same chain states and iteration counter, so every
(chain, SNP) draw uses the same counter-based uniforms.  Bounds, written
here and checked:
  * right-hand sides: max |rhs_fp8 - rhs_fp64| <= 1e-5 x max |rhs_fp64|;
  * conditional means of the effect draws: within 1e-3 conditional standard
    deviations;
  * class draws: identical for every (chain, SNP) whose decision margin
    (distance of its uniform from the nearest FP64 cumulative class
    probability) is at least TAU = 1e-4; disagreements below TAU are listed
    and allowed;
  * residuals after the subset's update: yadj = y - mu - X g to 1e-5
    relative, recomputed in FP64 on the host."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, precision, synth

pytestmark = pytest.mark.gpu

TAU = 1e-4

CASES = {
    "c3": dict(spec=synth.SynthSpec(n=20000, p=4000, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7, ncausal=16,
                                    h2=0.5, seed=303),
               opts=dict(method="BayesCpi", blocksize=2000), incl=0.01,
               pi=lambda ng: np.array([[0.99, 0.01]] * ng)),
    "c5": dict(spec=synth.SynthSpec(n=50000, p=2000, maf_lo=0.01, maf_hi=0.5, ld_block=100, rho=0.8, ncausal=10,
                                    h2=0.5, mixture=(1e-4, 1e-3, 1e-2), seed=505),
               opts=dict(method="BayesRc", nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2), ngroup=3, blocksize=1000),
               incl=0.01, pi=lambda ng: np.array([[0.97, 0.015, 0.01, 0.005], [0.95, 0.03, 0.015, 0.005],
                                                  [0.99, 0.006, 0.003, 0.001]])[:ng]),
}


def _job(G, y, opts, precision_, groups):
    cfg = make_config(G.shape[0], G.shape[1], JobOptions(numit=100, burnin=0, seed=4242, chains=16,
                                                         precision=precision_, scale_va=1.0, df_va=4.0,
                                                         scale_ve=1.0, df_ve=4.0, **opts))
    job = SodaJob(cfg)
    job.load_genotypes(G)
    job.load_pheno(y)
    if groups is not None:
        job.set_groups(groups)
    job.build_z()
    job.init_chains()
    return job


@pytest.mark.parametrize("case", ["c3", "c5"])
def test_fp8_tensor_subset_against_fp64(gpu_lib, case):
    cs = CASES[case]
    spec = cs["spec"]
    G, y, _ = synth.make(spec)
    groups = synth.annotation_groups(spec.p) if cs["opts"]["method"] == "BayesRc" else None
    job8 = _job(G, y, cs["opts"], "fp8", groups)
    job64 = _job(G, y, cs["opts"], "fp64", groups)
    nm = job64.cfg.nmix
    mix = [job64.cfg.mix[k] for k in range(nm)]
    vare = 0.5 * float(np.var(y))
    states = [precision.sparse_state(G, y, None, nm, mix, 1.0, vare, cs["incl"], cs["pi"](job64.cfg.ngroup), groups,
                                     seed=1000 + c, naind=job64.cfg.blocksize) for c in range(16)]
    try:
        res = precision.conditional_check(job8, job64, G, y, 0, 7, states, groups=groups, tau=TAU)
    finally:
        job8.close()
        job64.close()
    print(case, {k: v for k, v in res.items() if k != "disagreements"})
    assert res["rhs_max_abs_err_over_max"] <= 1e-5, res
    assert res["cond_mean_max_err_in_sd"] <= 1e-3, res
    assert res["disagreements_above_tau"] == 0, res.get("disagreements")
    assert res["residual_identity_rel_err"] <= 1e-5, res
