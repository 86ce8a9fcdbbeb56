"""The oracle's random-number layer: Philox known answers, the reference's
xoroshiro128+ streams and the distribution transforms."""
import numpy as np
import pytest
from scipy import stats

M64 = (1 << 64) - 1


def _xo_next(s):
    s1, s2 = s
    r = (s1 + s2) & M64
    s2 ^= s1
    s1 = (((s1 << 55) | (s1 >> 9)) & M64) ^ s2 ^ ((s2 << 14) & M64)
    s2 = ((s2 << 36) | (s2 >> 28)) & M64
    s[0], s[1] = s1, s2
    return r


def _xo_jump(s):
    a = b = 0
    for jm in (0xBEAC0467EBA5FACB, 0xD86B048B86AA9922):
        for bit in range(64):
            if jm >> bit & 1:
                a ^= s[0]
                b ^= s[1]
            _xo_next(s)
    s[0], s[1] = a, b


def _unit(x):
    bits = 0x3FF0000000000000 | (x >> 12)
    return float(np.frombuffer(np.uint64(bits).tobytes(), dtype=np.float64)[0]) - 1.0


def test_philox_known_answers(oracle_mod):
    # Random123 kat_vectors, philox4x32_10
    O = oracle_mod
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("seed,stream", [(123456789, 0), (123456789, 3), (-77, 1)])
def test_reference_streams(oracle_mod, seed, stream):
    """rng_zigset: stream k is (|seed|, |seed|+1) jumped k+1 times; values map
    u64 -> [0,1) as rng_int64_to_real64 (parallelrng.f90:54-149, 242-249)."""
    a = abs(seed)
    s = [a, a + 1]
    for _ in range(stream + 1):
        _xo_jump(s)
    want = [_unit(_xo_next(s)) for _ in range(64)]
    got = oracle_mod.ref_uniforms(seed, stream, 64)
    assert np.array_equal(np.array(want), got)


def test_counter_uniforms_layout(oracle_mod):
    """Counter stream: Philox(ctr={iter, slot, purpose, chain<<20 | call}, key=seed);
    each call yields two 64-bit words (x1:x0, x3:x2)."""
    O = oracle_mod
    seed = 0x1234_5678_9ABC
    got = O.counter_uniforms(seed, 2, 7, 99, 1, 6)
    key = [seed & 0xFFFFFFFF, seed >> 32]
    want = []
    for call in range(3):
        x = O.philox([7, 99, 1, (2 << 20) | call], key)
        want += [_unit((x[1] << 32) | x[0]), _unit((x[3] << 32) | x[2])]
    assert np.array_equal(got, np.array(want))
    assert np.all((got >= 0) & (got < 1))


@pytest.mark.parametrize("mode", [0, 1])
def test_normal_moments(oracle_mod, mode):
    x = oracle_mod.sample(1, mode, 99, 200000, 3.0, 2.0)
    assert abs(x.mean() - 3.0) < 0.02
    assert abs(x.std() - 2.0) < 0.02
    assert stats.kstest((x - 3.0) / 2.0, "norm").pvalue > 1e-4


@pytest.mark.parametrize("shape", [0.4, 1.0, 4.5, 250.0])
def test_gamma_moments(oracle_mod, shape):
    x = oracle_mod.sample(2, 0, 7, 100000, shape, 2.0)
    assert abs(x.mean() / (shape * 2.0) - 1) < 0.02
    assert stats.kstest(x, "gamma", args=(shape, 0, 2.0)).pvalue > 1e-4


def test_scaled_inverse_chi_square(oracle_mod):
    dof, scale = 10.0, 3.0
    x = oracle_mod.sample(3, 0, 5, 100000, dof, scale)
    assert abs(x.mean() / (dof * scale / (dof - 2)) - 1) < 0.02
    # 1/x ~ gamma(dof/2, 2/(dof*scale))
    assert stats.kstest(1.0 / x, "gamma", args=(dof / 2, 0, 2.0 / (dof * scale))).pvalue > 1e-4


def test_dirichlet(oracle_mod):
    x = oracle_mod.sample(4, 0, 3, 20000, 4, 2.5)
    assert np.allclose(x.sum(axis=1), 1.0, atol=1e-12)
    assert np.allclose(x.mean(axis=0), 0.25, atol=0.01)


def test_precision_module_philox_matches_oracle(oracle_mod):
    """The numpy Philox of sodabayes_gb300.precision (class-draw uniforms for
    the decision-margin analysis) gives the oracle's counter uniforms."""
    import ctypes as C

    from sodabayes_gb300 import precision as P
    L = oracle_mod.lib()
    for seed, ch, it, slot in [(4242, 0, 7, 0), (4242, 3, 7, 1999), (77, 15, 120, 499999), (2 ** 40 + 5, 2, 1, 12)]:
        out = np.empty(1)
        L.oracle_counter_uniforms(seed, ch, it, slot, 1, 1, out.ctypes.data_as(C.POINTER(C.c_double)))
        assert P.class_uniform(seed, ch, it, np.array([slot]), fp32=False)[0] == out[0]
        u32 = P.class_uniform(seed, ch, it, np.array([slot]), fp32=True)[0]
        assert 0.0 < u32 < 1.0 and abs(u32 - out[0]) <= 2.0 ** -24


def test_class_cumulative_two_classes():
    """BayesC class probability (models.f90:362-377) against the closed form
    of the two-class case, P(class 2) = 1 / (1 + exp(s1 - s2))."""
    from sodabayes_gb300 import precision as P
    rhs, zz, vare, gp = np.array([-3.0, 0.0, 0.7, 25.0]), 900.0, 2.0, np.array([0.0, 0.01])
    logp = np.log(np.array([[0.99, 0.01]] * 4))
    cum = P.class_cumulative(rhs, zz, vare, gp, logp)
    s2 = -0.5 * (np.log(gp[1] * zz / vare + 1.0) - rhs * (rhs / (zz + vare / gp[1])) / vare) + logp[:, 1]
    p2 = 1.0 / (1.0 + np.exp(logp[:, 0] - s2))
    assert np.allclose(cum[:, 0], 1.0 - p2, rtol=1e-12, atol=1e-15)
    assert np.allclose(cum[:, 1], 1.0)
