"""The subset-size autotuner of batched analyses (sodagpu_autotune_batch),
on the CPU: it needs no GPU.  Checked: the subset sizes share one step count
and stay within the cap; the choice is the least modelled time among the
step counts the tuner considers, recomputed here from the documented model;
more iterations favour fewer, larger subsets only while the per-step cost
dominates; bad arguments are refused."""
import math

import numpy as np
import pytest

from sodabayes_gb300 import SodaGpuError, autotune_batch

MODEL = (30.0, 2.6e12, 1.0, 4.0, 5e13, 6e11)


def _cost(n, p, iters, cap, S, m=MODEL):
    per_iter, build = S * m[0] * 1e-6, 0.0
    for nj, pj in zip(n, p):
        N = min(cap, math.ceil(pj / S))
        per_iter += 2.0 * (nj * pj * m[2] + pj * (N + 1.0) / 2.0 * m[3]) / m[1]
        build += pj * (nj * N / m[4] + N * N / (3.0 * m[5]))
    return iters * per_iter + build


def _config4_like(k=32, seed=4):
    rng = np.random.default_rng(seed)
    n = rng.integers(500, 20001, size=k)
    p = rng.integers(10000, 200001, size=k)
    return n, p


def test_sizes_share_one_step_count_and_respect_the_cap(gpu_lib):
    n, p = _config4_like()
    for cap in (256, 1000, 2000):
        bs, steps, secs = autotune_batch(n, p, 2000, max_blocksize=cap)
        assert np.all(bs >= 1) and np.all(bs <= cap)
        nb = -(-p // bs)
        assert steps == int(nb.max())
        S = int(math.ceil(p.max() / bs[int(np.argmax(p))]))
        assert np.all(bs == np.minimum(cap, -(-p // S)))
        assert secs == pytest.approx(_cost(n, p, 2000, cap, S), rel=1e-9)


def test_choice_is_the_least_modelled_time(gpu_lib):
    n, p = _config4_like(12, seed=9)
    for iters in (1, 50, 2000):
        bs, steps, secs = autotune_batch(n, p, iters, max_blocksize=2000)
        s_lo = max(1, int(max(-(-pj // 2000) for pj in p)))
        cands, S = [], s_lo
        while S <= p.max():
            cands.append(S)
            nx = S + max(1, S // 16)
            S = p.max() if (nx > p.max() and S < p.max()) else nx
        best = min(_cost(n, p, iters, 2000, S) for S in cands)
        assert secs == pytest.approx(best, rel=1e-12)


def test_short_runs_prefer_small_subsets(gpu_lib):
    """The Z build grows with the subset size and is paid once: for a short
    run the tuner picks smaller subsets than for a long one."""
    n, p = _config4_like(8, seed=3)
    bs_short, _, _ = autotune_batch(n, p, 5, max_blocksize=2000)
    bs_long, _, _ = autotune_batch(n, p, 5000, max_blocksize=2000)
    assert bs_short.sum() < bs_long.sum()


def test_bad_arguments(gpu_lib):
    with pytest.raises(SodaGpuError):
        autotune_batch([100], [0], 10)
    with pytest.raises(SodaGpuError):
        autotune_batch([100] * 65, [1000] * 65, 10)
    with pytest.raises(SodaGpuError):
        autotune_batch([100], [1000], 0)
    with pytest.raises(SodaGpuError):
        autotune_batch([100], [1000], 10, model=[1, 2, 3, 4, 5, 0])
