"""The host mirror of useroptions.f90's parsing rules (make_config)."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, make_config
from sodabayes_gb300._abi import fround


def test_float_options_round_through_real():
    # cast_float reads a default REAL (utilities.f90:168-171)
    cfg = make_config(10, 20, JobOptions(method="BayesC", pi=0.99, scale_va=0.01, df_va=4.5, blocksize=5))
    assert cfg.pizero == float(np.float32(0.99)) and cfg.pizero != 0.99
    assert cfg.scale_va == float(np.float32(0.01))
    assert cfg.df_va == 4.5


@pytest.mark.parametrize("method,nmix,mix0,mix1", [("BayesA", 1, 0.0, 0.0), ("BayesB", 2, 0.0, 0.0),
                                                   ("BayesC", 2, 0.0, 1.0), ("BayesCpi", 2, 0.0, 1.0)])
def test_nmix_and_mix_per_method(method, nmix, mix0, mix1):
    # parse_nmix / parse_priors (useroptions.f90:387-398, 502-507)
    cfg = make_config(10, 20, JobOptions(method=method, nmix=7, mix=(0, 1, 2, 3, 4, 5, 6), blocksize=5))
    assert cfg.nmix == nmix
    assert (cfg.mix[0], cfg.mix[1]) == (mix0, mix1)


def test_bayesr_mix_and_alpha():
    cfg = make_config(10, 20, JobOptions(method="BayesR", nmix=4, mix=(0, 1e-4, 1e-3, 1e-2), alpha=(1.0,),
                                         blocksize=5))
    assert list(cfg.mix)[:4] == [fround(v) for v in (0, 1e-4, 1e-3, 1e-2)]
    assert list(cfg.alpha)[:4] == [1.0] * 4
    with pytest.raises(ValueError):
        make_config(10, 20, JobOptions(method="BayesR", nmix=4, mix=(0, 1), blocksize=5))
    with pytest.raises(ValueError):
        make_config(10, 20, JobOptions(method="BayesR", nmix=3, mix=(0, 1, 2), alpha=(1, 2), blocksize=5))


def test_method_names_and_pi_range():
    assert make_config(10, 20, JobOptions(method="bayesrc", nmix=2, mix=(0, 1), blocksize=5)).method == 6
    with pytest.raises(ValueError):
        make_config(10, 20, JobOptions(method="BayesZ", blocksize=5))
    with pytest.raises(ValueError):
        make_config(10, 20, JobOptions(method="BayesB", pi=1.0, blocksize=5))


def test_soda_off_runs_the_regular_sampler():
    """blocksize <= 1 switches SODA off (soda.f90:418-421): the regular sampler
    (models.f90:607-962) runs, with one nominal subset of every SNP."""
    cfg = make_config(10, 20, JobOptions(method="BayesC", nthreads=1))
    assert cfg.sampler == 1 and (cfg.blocksize, cfg.nblocks, cfg.blockt) == (20, 1, 1)
