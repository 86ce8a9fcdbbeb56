"""Reproducibility: two contexts with the same configuration and seed give
bit-identical augmenting matrices and chain states (no floating-point
atomics; every split and segment sum is added in a fixed order), for the
FP64 path and for the 16-chain FP8 tensor-core path."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,chains", [("fp64", 1), ("fp8", 16)])
def test_same_seed_same_chain(gpu_lib, precision, chains):
    spec = synth.SynthSpec(n=1000, p=1700, ld_block=25, rho=0.6, ncausal=40, h2=0.5, mean=10.0, seed=33)
    G, y, _ = synth.make(spec)
    cfg = make_config(spec.n, spec.p, JobOptions(method="BayesCpi", pi=0.95, numit=100, burnin=1, blocksize=300,
                                                 seed=4242, precision=precision, chains=chains, scale_va=0.05,
                                                 df_va=4.0, scale_ve=0.5, df_ve=4.0))
    out = []
    for _ in range(2):
        with SodaJob(cfg) as job:
            job.load_genotypes(G)
            job.load_pheno(y)
            job.build_z()
            xa, xxd, _ = job.z()
            job.init_chains()
            job.run(3)
            out.append((xa, xxd, [job.state(c) for c in (0, chains - 1)]))
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][2], out[1][2]):
        for k in ("g", "cls", "yadj", "yaadj", "vara_s"):
            assert np.array_equal(a[k], b[k]), k
        for k in ("mu", "vare", "vara"):
            assert a[k] == b[k], k


def test_same_seed_same_chain_tensor_core_many_units(gpu_lib):
    """A shape where every CTA of the tensor-core kernels cycles several times
    through its code ring (subsets of 2000 SNPs, n = 6000): a slot refilled by
    the next bulk copy before its readers are done would show here as chains
    that part within a few iterations."""
    spec = synth.SynthSpec(n=6000, p=12000, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7, ncausal=60, h2=0.5,
                           seed=8)
    G, y, _ = synth.make(spec)
    cfg = make_config(spec.n, spec.p, JobOptions(method="BayesCpi", numit=100, burnin=0, blocksize=2000, seed=99,
                                                 precision="fp8", chains=16, scale_va=1.0, df_va=4.0,
                                                 scale_ve=float(np.var(y)) / 2, df_ve=4.0))
    out = []
    for _ in range(2):
        with SodaJob(cfg) as job:
            job.load_genotypes(G)
            job.load_pheno(y)
            job.build_z()
            job.init_chains()
            job.run(5)
            out.append([job.state(c) for c in range(16)])
    for c in range(16):
        for k in ("g", "cls", "yadj", "yaadj"):
            assert np.array_equal(out[0][c][k], out[1][c][k]), (c, k)
