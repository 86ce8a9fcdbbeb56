"""The oracle's Z-build building blocks against independent numpy algebra."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, make_config, synth


def _spd(n, rng, rank=None):
    A = rng.standard_normal((n, rank or n))
    return A @ A.T + (0 if rank else n * np.eye(n))


def test_cholesky_pd_matches_numpy(oracle_mod):
    rng = np.random.default_rng(0)
    A = _spd(40, rng)
    U, st = oracle_mod.cholesky_pd(A)
    assert st == 0
    assert np.allclose(U, np.linalg.cholesky(A).T, rtol=1e-12, atol=1e-10)


def test_cholesky_pd_reports_failing_row(oracle_mod):
    A = np.diag([4.0, 1.0, 9.0])
    A[1, 2] = A[2, 1] = 3.0          # row 2 becomes 9 - 9 = 0
    U, st = oracle_mod.cholesky_pd(A)
    assert st == 3
    A2 = np.diag([1.0, -1.0])
    _, st2 = oracle_mod.cholesky_pd(A2)
    assert st2 == -1                 # bad diagonal


def test_cholesky_psd_rank_and_reconstruction(oracle_mod):
    rng = np.random.default_rng(1)
    n, r = 30, 12
    A = _spd(n, rng, rank=r)
    F, piv, rank, st = oracle_mod.cholesky_psd(A)
    assert st == 0 and rank == r
    U = np.triu(F)[:rank, :]
    P = np.asarray(piv) - 1
    assert np.allclose(U.T @ U, A[np.ix_(P, P)], rtol=1e-9, atol=1e-8 * np.abs(A).max())


def test_power_method_matches_eigvalsh(oracle_mod):
    rng = np.random.default_rng(2)
    A = _spd(25, rng)
    lam, its = oracle_mod.power_method(A, rng.uniform(size=25), 100000)
    assert abs(lam / np.linalg.eigvalsh(A)[-1] - 1) < 1e-12


def test_gram_is_exact_centred_product(oracle_mod):
    """xxproduct's popcount Gram (soda.f90:520-556) equals X'X of the centred genotypes."""
    spec = synth.SynthSpec(n=333, p=64, seed=3)
    G, y, _ = synth.make(spec)
    G[:, 5] = 0   # monomorphic column -> zero row/column
    cfg = make_config(333, 64, JobOptions(method="BayesC", blocksize=32))
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    A = o.gram(np.arange(64))
    X = synth.centred(G)
    assert np.allclose(A, X.T @ X, rtol=1e-12, atol=1e-9)
    assert np.all(A[5] == 0) and np.all(A[:, 5] == 0)


@pytest.mark.parametrize("opts", [dict(blocksize=100), dict(nblocks=7), dict(blocksize=500)])
def test_augmenting_identity(oracle_mod, opts):
    """U_b'U_b + X_b'X_b = d_b I for every subset (soda.f90:484-491)."""
    n, p = 250, 480
    G, y, _ = synth.make(synth.SynthSpec(n=n, p=p, ld_block=20, rho=0.6, seed=9))
    cfg = make_config(n, p, JobOptions(method="BayesC", seed=5, **opts))
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    assert o.build_z() == 0
    xa, xxd, skip = o.z()
    X = synth.centred(G)
    ls = 0
    for b in range(cfg.nblocks):
        N = cfg.blocksize if b < cfg.blockt else cfg.blocksize - 1
        N = min(N, p - ls)
        Xb = X[:, ls:ls + N]
        U = xa[:N, ls:ls + N]
        assert np.allclose(np.tril(U, -1), 0)
        resid = U.T @ U + Xb.T @ Xb - xxd[b] * np.eye(N)
        assert np.abs(resid).max() < 1e-9 * xxd[b]
        assert abs(xxd[b] - (np.linalg.eigvalsh(Xb.T @ Xb)[-1] + np.float32(0.001))) < 1e-9 * xxd[b]
        ls += N
    assert ls == p
