"""GPU sampler (libsodagpu.so, through the C ABI) against the CPU oracle fed
the same counter-based draws.

Tolerances: the FP64 mode must reproduce the oracle's conditional draws to
1e-10 relative after one iteration (the reference-faithful bound), 1e-9
after a dozen iterations (rounding differences of the GPU's tree reductions
compound through the chain), with identical class indicators.  The Z build
matches to 1e-12 relative in d and 1e-9 relative (to the largest entry) in
the factor.  The reduced-precision modes are bounded against FP64."""
import numpy as np
import pytest

from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth

pytestmark = pytest.mark.gpu

N, P = 320, 900
GROUPS = (np.arange(P) % 3 + 1).astype(np.int32)


@pytest.fixture(scope="module")
def data():
    G, y, b = synth.make(synth.SynthSpec(n=N, p=P, ld_block=25, rho=0.5, ncausal=25, h2=0.5, mean=30.0, seed=21))
    return G, y, b


def _opts(method, **kw):
    base = dict(method=method, pi=0.99, numit=100, burnin=3, thin=2, blocksize=150, seed=987,
                scale_va=0.02, df_va=4.0, scale_ve=0.02, df_ve=4.0, precision="fp64")
    if method in ("BayesR", "BayesRc"):
        base.update(nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2))
    if method == "BayesRc":
        base.update(ngroup=3)
    base.update(kw)
    return JobOptions(**base)


def _pair(oracle_mod, data, opts, permvec=None, d_offset=0.0, codes=None):
    G, y, _ = data
    G = G if codes is None else codes
    cfg = make_config(G.shape[0], G.shape[1], opts)
    job = SodaJob(cfg)
    job.load_genotypes(G)
    job.load_pheno(y[:G.shape[0]])
    o = oracle_mod.Oracle(cfg)
    o.load_genotypes(G)
    o.load_pheno(y[:G.shape[0]])
    if cfg.method == 6:
        job.set_groups(GROUPS[:G.shape[1]])
        o.set_groups(GROUPS[:G.shape[1]])
    if d_offset:
        job.set_d_offset(d_offset)
    nsk_g = job.build_z(permvec)
    nsk_o = o.build_z(permvec, 0, d_offset)
    assert nsk_g == nsk_o
    job.init_chains()
    o.init_chains()
    return job, o


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


def _compare_state(job, o, tol, chain=0):
    sg, so = job.state(chain), o.state(chain)
    assert np.array_equal(sg["cls"], so["cls"])
    assert _rel(sg["g"], so["g"]) <= tol
    assert _rel(sg["yadj"], so["yadj"]) <= tol
    assert _rel(sg["yaadj"], so["yaadj"]) <= tol
    assert _rel(sg["vara_s"], so["vara_s"]) <= tol or np.all(so["vara_s"] == 0)
    for k in ("mu", "vare", "vara"):
        assert abs(sg[k] - so[k]) <= tol * max(1e-300, abs(so[k])), k
    assert sg["included"] == so["included"]


@pytest.mark.parametrize("method", ["BayesA", "BayesB", "BayesC", "BayesCpi", "BayesR", "BayesRc"])
def test_fp64_chain_matches_oracle(gpu_lib, oracle_mod, data, method):
    job, o = _pair(oracle_mod, data, _opts(method))
    # Z build: frequencies exactly, d and the factor to rounding
    assert np.array_equal(job.freq(), o.freq())
    xg, dg, sg = job.z()
    xo, do, so = o.z()
    assert np.all(np.abs(dg / do - 1) <= 1e-12)
    assert _rel(xg, xo) <= 1e-9
    assert np.array_equal(sg, so)
    _compare_state(job, o, 1e-12)          # initialisation (models.f90:56-128)
    rows_g, rows_o = [], []
    job.run(1, trace=lambda r: rows_g.append((r.rep, r.included, r.mu, r.vare, r.vara, list(r.snpindist))))
    o.run(1, trace=lambda r: rows_o.append((r.rep, r.included, r.mu, r.vare, r.vara, list(r.snpindist))))
    _compare_state(job, o, 1e-10)
    job.run(11, trace=lambda r: rows_g.append((r.rep, r.included, r.mu, r.vare, r.vara, list(r.snpindist))))
    o.run(11, trace=lambda r: rows_o.append((r.rep, r.included, r.mu, r.vare, r.vara, list(r.snpindist))))
    _compare_state(job, o, 1e-9)
    assert len(rows_g) == len(rows_o) == 6
    for a, b in zip(rows_g, rows_o):
        assert a[0] == b[0] and a[1] == b[1] and a[5] == b[5]
        assert np.allclose(a[2:5], b[2:5], rtol=1e-9, atol=0)
    rg, ro = job.results(), o.results()
    assert _rel(rg["gstore"], ro["gstore"]) <= 1e-9
    assert np.array_equal(rg["indiststore"], ro["indiststore"])
    for k in ("mu_store", "vare_store", "vara_store", "included_store"):
        assert abs(rg[k] - ro[k]) <= 1e-9 * max(1e-300, abs(ro[k])), k
    assert np.allclose(rg["snpstore"], ro["snpstore"], rtol=1e-12)
    assert np.allclose(rg["pstore"], ro["pstore"], rtol=1e-9)
    assert np.allclose(rg["varstore"], ro["varstore"], rtol=1e-9)
    if method in ("BayesA", "BayesB"):
        assert _rel(rg["vara_sstore"], ro["vara_sstore"]) <= 1e-9
    job.close()


def test_multichain_chain0_is_the_single_chain(gpu_lib, data):
    G, y, _ = data
    out = []
    for C in (1, 4):
        with SodaJob(make_config(N, P, _opts("BayesR", chains=C))) as job:
            job.load_genotypes(G)
            job.load_pheno(y)
            job.build_z()
            job.init_chains()
            job.run(8)
            out.append([job.state(c) for c in range(C)])
    # same draws; the kernels of different chain counts may round differently
    assert np.array_equal(out[0][0]["cls"], out[1][0]["cls"])
    assert _rel(out[1][0]["g"], out[0][0]["g"]) <= 1e-12
    assert _rel(out[1][0]["yadj"], out[0][0]["yadj"]) <= 1e-12
    # the other chains are different draws
    assert not np.array_equal(out[1][1]["g"], out[1][0]["g"])


def test_multichain_matches_oracle_chains(gpu_lib, oracle_mod, data):
    job, o = _pair(oracle_mod, data, _opts("BayesCpi", chains=2))
    job.run(5)
    o.run(5)
    for c in range(2):
        _compare_state(job, o, 1e-9, chain=c)


@pytest.mark.parametrize("method", ["BayesCpi", "BayesA"])
def test_pivoted_fallback_matches_oracle(gpu_lib, oracle_mod, data, method):
    """d pushed below lambda_max: both take choleskyPSD and skip the same SNPs
    (soda.f90:492-510), then run the single-site updates (models.f90:178-193, 433-495)."""
    job, o = _pair(oracle_mod, data, _opts(method), d_offset=-40.0)
    xg, dg, sg = job.z()
    xo, do, so = o.z()
    assert so.sum() > 0 and np.array_equal(sg, so)
    assert _rel(xg, xo) <= 1e-8
    job.run(4)
    o.run(4)
    _compare_state(job, o, 1e-8)


def test_random_blocks_and_nblocks_layout(gpu_lib, oracle_mod, data):
    """-rblocks permutation (utilities.f90:588-607) and -nblocks sizing with
    blockt < nblocks (soda.f90:410-412)."""
    opts = _opts("BayesC", blocksize=0, nblocks=7)
    cfg = make_config(N, P, opts)
    assert cfg.blockt < cfg.nblocks
    o0 = oracle_mod.Oracle(cfg)
    perm = o0.permutate()
    assert sorted(perm.tolist()) == list(range(1, P + 1))
    job, o = _pair(oracle_mod, data, opts, permvec=perm)
    job.run(6)
    o.run(6)
    _compare_state(job, o, 1e-9)


def test_residual_recalibration(gpu_lib, oracle_mod, data):
    job, o = _pair(oracle_mod, data, _opts("BayesR", recal_every=3))
    job.run(7)
    o.run(7)
    _compare_state(job, o, 1e-9)


def test_bed_input_and_edge_columns(gpu_lib, oracle_mod):
    """PLINK bed payload decodes on the device like load_geno, including
    missing calls and monomorphic SNPs; ragged n (not a multiple of 4)."""
    rng = np.random.default_rng(4)
    n, p = 203, 120
    raw = rng.integers(0, 4, size=(p, n)).astype(np.uint8)
    raw[7] = 0                    # monomorphic (all 00)
    raw[8] = 3                    # monomorphic (all 11)
    raw[9, :50] = 1               # many missing calls
    rec = (n + 3) // 4
    pad = np.zeros((p, rec * 4), dtype=np.uint8)
    pad[:, :n] = raw
    q = pad.reshape(p, rec, 4)
    bed = (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)
    codes = oracle_mod.decode_bed(bed, n, p)
    y = rng.standard_normal(n) + 5
    cfg = make_config(n, p, _opts("BayesCpi", blocksize=40))
    with SodaJob(cfg) as job:
        job.load_genotypes(bed=bed)
        job.load_pheno(y)
        o = oracle_mod.Oracle(cfg)
        o.load_genotypes(codes)
        o.load_pheno(y)
        assert np.array_equal(job.freq(), o.freq())
        assert job.build_z() == o.build_z()
        job.init_chains()
        o.init_chains()
        job.run(5)
        o.run(5)
        _compare_state(job, o, 1e-9)
        # monomorphic columns are zero (utilities.f90:528-529): no genomic value
        e = np.zeros(p)
        e[7], e[8] = 1.0, -2.0
        assert np.all(job.compute_dgv(0.0, e) == 0.0)


def test_invalid_codes_are_rejected(gpu_lib):
    from sodabayes_gb300 import SodaGpuError
    G = np.zeros((16, 10), dtype=np.int8)
    G[3, 4] = 3
    with SodaJob(make_config(16, 10, _opts("BayesC", blocksize=5))) as job:
        with pytest.raises(SodaGpuError):
            job.load_genotypes(G)


def test_compute_dgv_matches_oracle(gpu_lib, oracle_mod, data):
    job, o = _pair(oracle_mod, data, _opts("BayesC"))
    eff = np.random.default_rng(1).standard_normal(P) * 0.1
    assert np.allclose(job.compute_dgv(12.5, eff), o.compute_dgv(12.5, eff), rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("prec", ["fp32", "fp8"])
def test_reduced_precision_tracks_fp64(gpu_lib, data, prec):
    """Same draws, reduced-precision dot products: after three iterations the
    class indicators agree almost everywhere and the effects stay close."""
    G, y, _ = data
    st = {}
    for pr in ("fp64", prec):
        with SodaJob(make_config(N, P, _opts("BayesCpi", precision=pr, chains=2))) as job:
            job.load_genotypes(G)
            job.load_pheno(y)
            job.build_z()
            job.init_chains()
            job.run(3)
            st[pr] = job.state(1)
    agree = np.mean(st[prec]["cls"] == st["fp64"]["cls"])
    assert agree >= 0.99
    same = st[prec]["cls"] == st["fp64"]["cls"]
    d = st[prec]["g"][same] - st["fp64"]["g"][same]
    assert np.sqrt(np.mean(d ** 2)) <= 1e-3 * np.sqrt(np.mean(st["fp64"]["g"] ** 2))


def test_augmenting_identity_mid_size(gpu_lib):
    """Size-independent property at a larger size (n=4000, p=12000, s=1000):
    U_b'U_b + X_b'X_b = d_b I for sampled subsets, d_b >= lambda_max."""
    n, p, s = 4000, 12000, 1000
    G, y, _ = synth.make(synth.SynthSpec(n=n, p=p, maf_lo=0.01, ld_block=50, rho=0.7, ncausal=100, seed=8))
    with SodaJob(make_config(n, p, _opts("BayesCpi", blocksize=s, precision="fp8"))) as job:
        job.load_genotypes(G)
        job.load_pheno(y)
        assert job.build_z() == 0
        xa, xxd, skip = job.z()
    X = synth.centred(G)
    for b in (0, 5, 11):
        Xb = X[:, b * s:(b + 1) * s]
        A = Xb.T @ Xb
        U = xa[:, b * s:(b + 1) * s]
        assert np.abs(U.T @ U + A - xxd[b] * np.eye(s)).max() <= 1e-9 * xxd[b]
        lam = np.linalg.eigvalsh(A)[-1]
        assert abs(xxd[b] - lam - np.float32(0.001)) <= 1e-10 * lam
