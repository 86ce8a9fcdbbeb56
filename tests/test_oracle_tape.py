"""Injected-draw tape on the CPU: a chain run on the reference's own
per-thread xoroshiro128+ streams (parallelrng.f90:100-149, OpenMP static
chunking of each subset for four threads, as in the reference's example runs)
records the uniforms of every draw site; a second oracle that takes its
uniforms from that tape must reproduce the chain bit for bit.  The same for a
counter-mode (Philox) chain."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, make_config, synth

N, P = 200, 600
GROUPS = (np.arange(P) % 3 + 1).astype(np.int32)


def _cfg(method):
    kw = dict(method=method, pi=0.95, numit=10, burnin=1, blocksize=100, seed=31337, precision="fp64",
              scale_va=0.05, df_va=4.0, scale_ve=0.5, df_ve=4.0)
    if method in ("BayesR", "BayesRc"):
        kw.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    if method == "BayesRc":
        kw.update(ngroup=3)
    return make_config(N, P, JobOptions(**kw))


def _oracle(O, cfg, G, y, mode, threads=1, z=None):
    """z: the Z of another oracle (the reference mode's power method starts from stream 0, so its d and
    U differ from a counter-mode build in the last bits, which the sampler amplifies)."""
    o = O.Oracle(cfg, rng_mode=mode, ref_threads=threads)
    o.load_genotypes(G)
    o.load_pheno(y)
    if cfg.method == 6:
        o.set_groups(GROUPS)
    if z is None:
        o.build_z()
    else:
        o.set_z(z[0], z[1])
    return o


@pytest.mark.parametrize("method", ["BayesA", "BayesB", "BayesC", "BayesCpi", "BayesR", "BayesRc"])
@pytest.mark.parametrize("mode", ["reference", "counter"])
def test_tape_replays_the_recorded_chain(oracle_mod, method, mode):
    O = oracle_mod
    G, y, _ = synth.make(synth.SynthSpec(n=N, p=P, ld_block=20, rho=0.5, ncausal=15, h2=0.5, mean=5.0, seed=8))
    cfg = _cfg(method)
    m = O.RNG_REFERENCE if mode == "reference" else O.RNG_COUNTER
    rec = _oracle(O, cfg, G, y, m, threads=4)
    tape = rec.record_tape(4)
    rec.init_chains()
    rec.run(3)
    play = _oracle(O, cfg, G, y, O.RNG_COUNTER, z=rec.z()[:2])
    play.play_tape(tape)
    play.init_chains()
    play.run(3)
    a, b = rec.state(), play.state()
    for k in ("g", "yadj", "yaadj", "vara_s"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["cls"], b["cls"])
    for k in ("mu", "vare", "vara"):
        assert a[k] == b[k], k
    # every iteration used its records: mu, sigma2_e and ra sites hold uniforms in (0, 1)
    sites = rec._lib.oracle_tape_sites(rec._o)
    t = tape.reshape(4, sites, -1)
    assert np.all(t[1:, 0, :2] > 0.0) and np.all(t[:, 2, 0] > 0.0)
    rec.close()
    play.close()


def test_tape_shorter_than_the_run_is_an_error(oracle_mod):
    O = oracle_mod
    G, y, _ = synth.make(synth.SynthSpec(n=N, p=P, ncausal=15, h2=0.5, seed=9))
    cfg = _cfg("BayesC")
    rec = _oracle(O, cfg, G, y, O.RNG_COUNTER)
    tape = rec.record_tape(2)
    rec.init_chains()
    rec.run(1)
    play = _oracle(O, cfg, G, y, O.RNG_COUNTER, z=rec.z()[:2])
    play.play_tape(tape)
    play.init_chains()
    play.run(1)
    assert np.array_equal(play.state()["g"], rec.state()["g"])
    with pytest.raises(RuntimeError):
        play.run(1)          # iteration 2 is past the tape
    rec.close()
    play.close()
