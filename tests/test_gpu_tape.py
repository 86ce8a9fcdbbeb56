"""Injected-draw mode on the GPU (sodagpu_set_tape).

1. A tape of the counter-based draws (recorded by the oracle in counter mode)
   replayed on the GPU gives the GPU's own counter-mode chain bit for bit:
   the tape path changes where the uniforms come from and nothing else.
2. The reference's own draws: the oracle replays the reference's per-thread
   xoroshiro128+ streams (parallelrng.f90:100-149) with the OpenMP static
   chunking of each subset for four threads, seeded like set_random_seed
   (utilities.f90:504-517) and after the Z build's draws from stream 0
   (soda.f90:390), and records every draw site's uniforms.  The GPU, fed that
   tape, must match the oracle's chain like the counter-mode parity tests:
   identical class indicators, 1e-10 relative after one iteration and 1e-9
   after three.  Both use the GPU's Z (the oracle's power method starts from
   stream 0, so its d differs from the GPU's in the last bits, and the
   factor's conditioning carries that into the draws)."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu

N, P = 320, 900
GROUPS = (np.arange(P) % 3 + 1).astype(np.int32)
METHODS = ["BayesA", "BayesB", "BayesC", "BayesCpi", "BayesR", "BayesRc"]


@pytest.fixture(scope="module")
def data():
    G, y, _ = synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.5, ncausal=25, h2=0.5, mean=30.0, seed=21))
    return G, y


def _cfg(method):
    kw = dict(method=method, pi=0.99, numit=100, burnin=1, thin=1, blocksize=150, seed=987654321,
              scale_va=0.02, df_va=4.0, scale_ve=0.02, df_ve=4.0, precision="fp64")
    if method in ("BayesR", "BayesRc"):
        kw.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    if method == "BayesRc":
        kw.update(ngroup=3)
    return make_config(N, P, JobOptions(**kw))


def _gpu(cfg, G, y, tape=None):
    job = SodaJob(cfg)
    job.load_genotypes(G)
    job.load_pheno(y)
    if cfg.method == 6:
        job.set_groups(GROUPS)
    job.build_z()
    if tape is not None:
        job.set_tape(tape)
    job.init_chains()
    return job


def _oracle(O, cfg, G, y, mode, z):
    o = O.Oracle(cfg, rng_mode=mode, ref_threads=4)
    o.load_genotypes(G)
    o.load_pheno(y)
    if cfg.method == 6:
        o.set_groups(GROUPS)
    o.build_z()            # consumes the Z build's draws (reference mode: stream 0)
    o.set_z(z[0], z[1])    # then sweeps on the GPU's Z
    return o


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


def _same(sg, so, tol):
    assert np.array_equal(sg["cls"], so["cls"])
    for k in ("g", "yadj", "yaadj"):
        assert _rel(sg[k], so[k]) <= tol, k
    assert _rel(sg["vara_s"], so["vara_s"]) <= tol or np.all(so["vara_s"] == 0)
    for k in ("mu", "vare", "vara"):
        assert abs(sg[k] - so[k]) <= tol * max(1e-300, abs(so[k])), k


@pytest.mark.parametrize("method", METHODS)
def test_counter_tape_reproduces_the_counter_chain(gpu_lib, oracle_mod, data, method):
    G, y = data
    cfg = _cfg(method)
    plain = _gpu(cfg, G, y)
    z = plain.z()[:2]
    o = _oracle(oracle_mod, cfg, G, y, oracle_mod.RNG_COUNTER, z)
    tape = o.record_tape(4)
    o.init_chains()
    o.run(3)
    taped = _gpu(cfg, G, y, tape)
    try:
        plain.run(3)
        taped.run(3)
        a, b = plain.state(), taped.state()
        for k in ("g", "yadj", "yaadj", "vara_s"):
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a["cls"], b["cls"])
        for k in ("mu", "vare", "vara"):
            assert a[k] == b[k], k
    finally:
        plain.close()
        taped.close()
        o.close()


@pytest.mark.parametrize("method", METHODS)
def test_reference_streams_fed_to_the_gpu(gpu_lib, oracle_mod, data, method):
    G, y = data
    cfg = _cfg(method)
    zjob = _gpu(cfg, G, y)
    z = zjob.z()[:2]
    zjob.close()
    o = _oracle(oracle_mod, cfg, G, y, oracle_mod.RNG_REFERENCE, z)
    tape = o.record_tape(4)      # filled as the oracle runs: run it first
    o.init_chains()
    want = [o.state()]
    o.run(1)
    want.append(o.state())
    o.run(2)
    want.append(o.state())
    o.close()
    job = _gpu(cfg, G, y, tape)
    try:
        _same(job.state(), want[0], 1e-12)        # chain initialisation (sigma2_e, yAadj)
        job.run(1)
        _same(job.state(), want[1], 1e-10)
        job.run(2)
        _same(job.state(), want[2], 1e-9)
        # past the tape's four iterations (0 .. 3) the GPU refuses to draw
        from sodabayes_gb300 import SodaGpuError
        with pytest.raises(SodaGpuError):
            job.run(1)
    finally:
        job.close()
