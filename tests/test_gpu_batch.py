"""Many analyses in one launch per kernel (sodagpu_batch_*): every job of a
batch must give what it gives on its own.

Jobs of uneven n and p (and, in one test, different methods) run first one
by one, then again, freshly set up, as one batch.  With the jobs' own rhs
splits (SODAGPU_BATCH_SOLO_SPLITS) the states after four iterations and the
posterior means are bit-identical.  With the default autotuned splits the
rhs partial sums are grouped differently: FP64 jobs then agree in every
class indicator and within 1e-10 relative.  The subset sizes come from the
batch autotuner (sodagpu_autotune_batch)."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaBatch, SodaGpuError, SodaJob, autotune_batch, make_config, synth

pytestmark = pytest.mark.gpu

SHAPES = [(300, 1500), (900, 4000), (1500, 2500), (2400, 6000)]


def _data():
    out = []
    for k, (n, p) in enumerate(SHAPES):
        spec = synth.SynthSpec(n=n, p=p, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7,
                               ncausal=max(5, p // 200), h2=0.1 + 0.15 * k, seed=4100 + k)
        G, y, _ = synth.make(spec)
        out.append((G, y))
    return out


@pytest.fixture(scope="module")
def data():
    return _data()


def _job(G, y, opts):
    job = SodaJob(make_config(G.shape[0], G.shape[1], opts))
    job.load_genotypes(G)
    job.load_pheno(y)
    job.build_z()
    job.init_chains()
    return job


def _opts(k, bs, method, precision, chains):
    return JobOptions(method=method, blocksize=int(bs), numit=100, burnin=1, seed=777 + 31 * k,
                      precision=precision, chains=chains, kernels="cuda_cores",
                      scale_va=1.0, df_va=4.0, scale_ve=1.0, df_ve=4.0)


def _snapshot(job):
    out = []
    for c in range(job.chains):
        st = job.state(c)
        out.append((st, job.results(c)))
    return out


def _run(data, methods, precision, chains, solo_splits, iters=4):
    n = [G.shape[0] for G, _ in data]
    p = [G.shape[1] for G, _ in data]
    bs, steps, _ = autotune_batch(n, p, 2000, max_blocksize=512)
    assert steps == max(-(-pj // bj) for pj, bj in zip(p, bs))
    alone = []
    for k, (G, y) in enumerate(data):
        job = _job(G, y, _opts(k, bs[k], methods[k], precision, chains))
        try:
            job.run(iters)
            alone.append(_snapshot(job))
        finally:
            job.close()
    jobs = [_job(G, y, _opts(k, bs[k], methods[k], precision, chains)) for k, (G, y) in enumerate(data)]
    try:
        with SodaBatch(jobs, solo_splits=solo_splits) as b:
            b.run(iters)
            ms, st = b.timings()
            assert st == steps and ms > 0
        together = [_snapshot(j) for j in jobs]
    finally:
        for j in jobs:
            j.close()
    return alone, together


def _results_equal(ra, rb, tol):
    for key in ra:
        va, vb = np.asarray(ra[key], dtype=np.float64), np.asarray(rb[key], dtype=np.float64)
        if tol == 0:
            assert np.array_equal(va, vb), key
        else:
            assert np.max(np.abs(va - vb)) <= tol * max(1e-300, np.max(np.abs(vb))), key


def test_batch_is_bit_identical_with_solo_splits_fp8_bayesb(gpu_lib, data):
    alone, together = _run(data, ["BayesB"] * 4, "fp8", 1, True)
    for a, t in zip(alone, together):
        for (sa, ra), (st, rt) in zip(a, t):
            for key in ("g", "cls", "vara_s", "yadj", "yaadj"):
                assert np.array_equal(sa[key], st[key]), key
            for key in ("mu", "vare", "vara", "included"):
                assert sa[key] == st[key], key
            _results_equal(ra, rt, 0)


def test_batch_mixed_methods_fp64_two_chains(gpu_lib, data):
    methods = ["BayesA", "BayesCpi", "BayesR", "BayesB"]
    alone, together = _run(data, methods, "fp64", 2, True)
    for a, t in zip(alone, together):
        for (sa, _), (st, _) in zip(a, t):
            assert np.array_equal(sa["g"], st["g"]) and np.array_equal(sa["cls"], st["cls"])
            assert np.array_equal(sa["yadj"], st["yadj"])
    # autotuned splits: another grouping of the rhs partial sums, FP64 rounding only
    alone, together = _run(data, methods, "fp64", 2, False)
    for a, t in zip(alone, together):
        for (sa, _), (st, _) in zip(a, t):
            assert np.array_equal(sa["cls"], st["cls"])
            for key in ("g", "yadj"):
                assert np.max(np.abs(sa[key] - st[key])) <= 1e-10 * max(1e-300, np.max(np.abs(sa[key]))), key


def test_batch_rejects_jobs_it_cannot_run(gpu_lib, data):
    G, y = data[0]
    a = _job(G, y, _opts(0, 500, "BayesB", "fp8", 1))
    b = _job(G, y, _opts(1, 500, "BayesB", "fp8", 2))
    tc = _job(G, y, JobOptions(method="BayesB", blocksize=500, numit=10, burnin=1, seed=5, precision="fp8",
                               chains=4, scale_va=1.0, df_va=4.0, scale_ve=1.0, df_ve=4.0))
    try:
        with pytest.raises(SodaGpuError):
            SodaBatch([a, b])            # different chain counts
        with pytest.raises(SodaGpuError):
            SodaBatch([a, tc])           # a job on the tensor-core kernels
        with pytest.raises(SodaGpuError):
            SodaBatch([a, a])            # the same job twice
    finally:
        for j in (a, b, tc):
            j.close()
