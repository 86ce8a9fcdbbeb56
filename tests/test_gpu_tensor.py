"""Tensor-core sweep (FP8 mode, 4/8/16 chains: tcgen05 genotype products with
bf16 hi/mid/lo splits) against the CUDA-core FP8 sweep, the FP64 sweep and a
host recomputation of the residuals.

Tolerances: the two FP8 sweeps compute the same FP32-accurate products in a
different summation order, so after one iteration their class indicators
agree on >= 99.9% of SNP x chain pairs and the effects to 1e-4 relative RMS;
against FP64 the bound of the reduced-precision modes applies (>= 99% of
classes, 1e-3 relative RMS).  The residual kept on the device must equal
y - mu - X g recomputed in FP64 to 1e-5 relative."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu

N, P, S = 1000, 1700, 300   # n not a multiple of 128, subsets of 300 and 299 SNPs
GROUPS = (np.arange(P) % 3 + 1).astype(np.int32)   # three annotation classes for BayesRc


@pytest.fixture(scope="module")
def data():
    return synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.6, ncausal=40, h2=0.5, mean=10.0, seed=33))


def _opts(**kw):
    base = dict(method="BayesCpi", pi=0.95, numit=100, burnin=2, thin=1, blocksize=S, seed=4242,
                scale_va=0.05, df_va=4.0, scale_ve=0.5, df_ve=4.0, precision="fp8")
    base.update(kw)
    return JobOptions(**base)


def _run(data, iters, d_offset=0.0, **kw):
    G, y, _ = data
    cfg = make_config(N, P, _opts(**kw))
    with SodaJob(cfg) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        if cfg.ngroup > 1:
            job.set_groups(GROUPS)
        if d_offset:
            job.set_d_offset(d_offset)
        job.build_z()
        job.init_chains()
        job.run(iters)
        return [job.state(c) for c in range(job.chains)]


def _agree(a, b):
    same = a["cls"] == b["cls"]
    d = a["g"][same] - b["g"][same]
    return np.mean(same), np.sqrt(np.mean(d ** 2)) / max(1e-300, np.sqrt(np.mean(b["g"] ** 2)))


@pytest.mark.parametrize("chains", [4, 8, 16])
def test_tensor_sweep_matches_cuda_core_sweep(gpu_lib, data, chains):
    tcs = _run(data, 1, chains=chains)
    ref = _run(data, 1, chains=chains, kernels="cuda_cores")
    for c in range(chains):
        agree, rel = _agree(tcs[c], ref[c])
        assert agree >= 0.999, (c, agree)
        assert rel <= 1e-4, (c, rel)
        assert abs(tcs[c]["vare"] - ref[c]["vare"]) <= 1e-4 * ref[c]["vare"]


@pytest.mark.parametrize("method", ["BayesA", "BayesB", "BayesC", "BayesR", "BayesRc"])
def test_tensor_sweep_every_method(gpu_lib, data, method):
    """Every model on the tensor-core path with 16 chains on shared genotypes
    (BayesRc: four-class mixtures in three annotation groups, the shape of the
    16-chain BayesRc analysis at a size the CUDA-core sweep checks quickly)."""
    kw = dict(method=method, chains=16, pi=0.95)
    if method in ("BayesR", "BayesRc"):
        kw.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    if method == "BayesRc":
        kw.update(ngroup=3)
    tcs = _run(data, 1, **kw)
    ref = _run(data, 1, kernels="cuda_cores", **kw)
    for c in range(16):
        agree, rel = _agree(tcs[c], ref[c])
        assert agree >= 0.999, (c, agree)
        assert rel <= 1e-3, (c, rel)
        assert abs(tcs[c]["vare"] - ref[c]["vare"]) <= 1e-3 * ref[c]["vare"]


def test_tensor_sweep_tracks_fp64(gpu_lib, data):
    tcs = _run(data, 3, chains=4)
    f64 = _run(data, 3, chains=4, precision="fp64")
    for c in range(4):
        agree, rel = _agree(tcs[c], f64[c])
        assert agree >= 0.99, (c, agree)
        assert rel <= 1e-3, (c, rel)


@pytest.mark.parametrize("chains", [4, 16])
def test_tensor_residual_is_consistent(gpu_lib, data, chains):
    """r = y - mu - X g after several iterations (recalibration every 1000)."""
    G, y, _ = data
    X = synth.centred(G)
    st = _run(data, 4, chains=chains)
    for c in (0, chains - 1):
        r_host = y - st[c]["mu"] - X @ st[c]["g"]
        r_dev = st[c]["yadj"][:N]
        assert np.max(np.abs(r_dev - r_host)) <= 1e-5 * np.max(np.abs(r_host)), c


def test_tensor_sweep_pivoted_fallback(gpu_lib, data):
    """Forced pivoted fallback (no triangular skipping in the ra update)."""
    Xb = synth.centred(data[0])[:, :S]
    off = -0.2 * np.linalg.eigvalsh(Xb.T @ Xb)[-1]
    tcs = _run(data, 1, chains=4, d_offset=off)
    ref = _run(data, 1, chains=4, d_offset=off, kernels="cuda_cores")
    for c in range(4):
        agree, rel = _agree(tcs[c], ref[c])
        assert agree >= 0.999, (c, agree)
        assert rel <= 1e-4, (c, rel)
        ya, yr = tcs[c]["yaadj"], ref[c]["yaadj"]
        assert np.max(np.abs(ya - yr)) <= 1e-4 * max(1e-300, np.max(np.abs(yr)))


def test_profile_counts_every_subset_kernel(gpu_lib, data):
    """sodagpu_profile_kernels records every launch of an iteration (rhs,
    draws and update of every subset)."""
    G, y, _ = data
    cfg = make_config(N, P, _opts(chains=16))
    with SodaJob(cfg) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        prof = job.profile_kernels(2)
    nb = cfg.nblocks
    assert prof["rhs"][1] == 2 * nb and prof["update"][1] == 2 * nb and prof["draw"][1] == 2 * nb
    assert prof["mu"][1] == 2 and prof["other"][1] == 2
    assert all(v[0] > 0.0 for v in prof.values())
