"""Seeded synthetic genotypes and phenotypes with the shapes of the benchmark
configurations (no public data set is involved).

Genotypes are Binomial(2, maf) codes.  With `ld_block > 1` each haplotype is a
thresholded latent Gaussian AR(1) process within blocks of `ld_block` SNPs, so
neighbouring SNPs are in LD; the individual's code is the sum of two
haplotypes.  Phenotypes are y = X b + e with X the centred/scaled genotypes
and e scaled so that var(Xb) / var(y) = h2.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SynthSpec:
    n: int
    p: int
    maf_lo: float = 0.05
    maf_hi: float = 0.5
    ld_block: int = 0
    rho: float = 0.0
    ncausal: int = 100
    h2: float = 0.5
    mixture: tuple = ()          # class variances (share of Va) for causal effects, e.g. (1e-4,1e-3,1e-2)
    mean: float = 0.0
    seed: int = 1


def _std_normal_quantile(p):
    from scipy.special import ndtri
    return ndtri(p)


def genotypes(spec: SynthSpec, rng: np.random.Generator) -> np.ndarray:
    """int8 codes, shape (n, p), Fortran order (one SNP per column)."""
    n, p = spec.n, spec.p
    maf = rng.uniform(spec.maf_lo, spec.maf_hi, size=p)
    G = np.empty((n, p), dtype=np.int8, order="F")
    if spec.ld_block <= 1 or spec.rho == 0.0:
        for j0 in range(0, p, 4096):
            j1 = min(p, j0 + 4096)
            G[:, j0:j1] = rng.binomial(2, maf[j0:j1], size=(n, j1 - j0)).astype(np.int8)
        return G
    thr = _std_normal_quantile(maf)
    s = np.sqrt(1.0 - spec.rho * spec.rho)
    L = spec.ld_block
    for j0 in range(0, p, L):
        j1 = min(p, j0 + L)
        codes = np.zeros((n, j1 - j0), dtype=np.int8)
        for _h in range(2):
            z = rng.standard_normal(n)
            for j in range(j0, j1):
                if j > j0:
                    z = spec.rho * z + s * rng.standard_normal(n)
                codes[:, j - j0] += (z < thr[j]).astype(np.int8)
        G[:, j0:j1] = codes
    return G


def centred(G: np.ndarray) -> np.ndarray:
    """xscale (utilities.f90:525-534) in float64."""
    n = G.shape[0]
    f = G.sum(axis=0, dtype=np.float64) / (2.0 * n)
    eps = np.finfo(np.float64).eps
    ok = (f >= eps) & (1.0 - f >= eps)
    sd = np.where(ok, np.sqrt(2.0 * f * (1.0 - f)), 1.0)
    return np.where(ok, (G - 2.0 * f) / sd, 0.0)


def phenotypes(G: np.ndarray, spec: SynthSpec, rng: np.random.Generator):
    """Returns (y, b): true effects b (length p) and y = mean + X b + e."""
    n, p = G.shape
    b = np.zeros(p)
    k = min(spec.ncausal, p)
    pos = rng.choice(p, size=k, replace=False)
    if spec.mixture:
        var = np.asarray(spec.mixture, dtype=np.float64)
        cls = rng.integers(0, len(var), size=k)
        b[pos] = rng.standard_normal(k) * np.sqrt(var[cls])
    else:
        b[pos] = rng.standard_normal(k)
    g = np.zeros(n)
    for j0 in range(0, p, 8192):
        j1 = min(p, j0 + 8192)
        if np.any(b[j0:j1]):
            g += centred(G[:, j0:j1]) @ b[j0:j1]
    vg = g.var()
    ve = vg * (1.0 - spec.h2) / spec.h2 if vg > 0 else 1.0
    y = spec.mean + g + rng.standard_normal(n) * np.sqrt(ve)
    return y, b


def make(spec: SynthSpec):
    rng = np.random.default_rng(spec.seed)
    G = genotypes(spec, rng)
    y, b = phenotypes(G, spec, rng)
    return G, y, b


# The five benchmark configurations, by their generator settings.
CONFIGS = {
    "c1": SynthSpec(n=1000, p=5000, maf_lo=0.05, maf_hi=0.5, ncausal=100, h2=0.5, seed=20260001),
    "c2": SynthSpec(n=5000, p=50000, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7, ncausal=1000, h2=0.4,
                    mixture=(1e-4, 1e-3, 1e-2), seed=20260002),
    "c3": SynthSpec(n=20000, p=500000, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7, ncausal=2000, h2=0.5,
                    seed=20260003),
    # BayesRc, 16 chains on shared genotypes: 100-SNP LD blocks, rho = 0.8, 5000 causal effects from the
    # non-zero mixture components, three annotation classes (annotation_groups)
    "c5": SynthSpec(n=50000, p=1000000, maf_lo=0.01, maf_hi=0.5, ld_block=100, rho=0.8, ncausal=5000, h2=0.5,
                    mixture=(1e-4, 1e-3, 1e-2), seed=20260005),
}


def annotation_groups(p: int, proportions=(0.1, 0.3, 0.6), seed: int = 20260105) -> np.ndarray:
    """SNP annotation classes 1..len(proportions) (the group file of BayesRc),
    in the given proportions, assigned at random positions."""
    rng = np.random.default_rng(seed)
    order = rng.permutation(p)
    grp = np.empty(p, dtype=np.int32)
    edges = np.round(np.cumsum((0.0,) + tuple(proportions)) * p).astype(np.int64)
    edges[-1] = p
    for g in range(len(proportions)):
        grp[order[edges[g]:edges[g + 1]]] = g + 1
    return grp


def make_device(spec: SynthSpec, device="cuda"):
    """The same generator on the GPU with torch, for the full-size workloads.

    Returns (codes, y, b): codes is an int8 torch tensor of shape (p, n) on
    `device` — SNP-major, i.e. the column-major (n, p) matrix the C ABI takes
    as SODAGPU_GENO_CODES — y and b are numpy arrays.  The random streams
    differ from make(); the distributions are the same."""
    import torch

    n, p = spec.n, spec.p
    gen = torch.Generator(device=device)
    gen.manual_seed(spec.seed)
    maf = torch.rand(p, generator=gen, device=device, dtype=torch.float64) * (spec.maf_hi - spec.maf_lo) + spec.maf_lo
    codes = torch.empty((p, n), dtype=torch.int8, device=device)
    if spec.ld_block <= 1 or spec.rho == 0.0:
        for j0 in range(0, p, 2048):
            j1 = min(p, j0 + 2048)
            u = torch.rand((j1 - j0, n, 2), generator=gen, device=device, dtype=torch.float32)
            codes[j0:j1] = (u < maf[j0:j1, None, None].float()).sum(dim=2).to(torch.int8)
    else:
        L = spec.ld_block
        nfull = p // L
        thr = torch.special.ndtri(maf).float()
        s = float(np.sqrt(1.0 - spec.rho * spec.rho))
        chunk = max(1, (1 << 27) // max(n, 1))      # LD blocks per pass (~128M latent values)
        for b0 in range(0, nfull, chunk):
            b1 = min(nfull, b0 + chunk)
            view = codes[b0 * L:b1 * L].view(b1 - b0, L, n)
            acc = torch.zeros((b1 - b0, L, n), dtype=torch.int8, device=device)
            for _h in range(2):
                z = torch.randn((b1 - b0, n), generator=gen, device=device)
                for t in range(L):
                    if t:
                        z = spec.rho * z + s * torch.randn((b1 - b0, n), generator=gen, device=device)
                    acc[:, t, :] += (z < thr[b0 * L + t:b1 * L:L, None]).to(torch.int8)
            view.copy_(acc)
        if nfull * L < p:   # ragged tail: independent SNPs
            j0 = nfull * L
            u = torch.rand((p - j0, n, 2), generator=gen, device=device)
            codes[j0:] = (u < maf[j0:, None, None].float()).sum(dim=2).to(torch.int8)
    # phenotype
    rng = np.random.default_rng(spec.seed + 1)
    b = np.zeros(p)
    k = min(spec.ncausal, p)
    pos = np.sort(rng.choice(p, size=k, replace=False))
    if spec.mixture:
        var = np.asarray(spec.mixture, dtype=np.float64)
        cls = rng.integers(0, len(var), size=k)
        b[pos] = rng.standard_normal(k) * np.sqrt(var[cls])
    else:
        b[pos] = rng.standard_normal(k)
    cols = codes[torch.as_tensor(pos, device=device)].double()             # (k, n)
    f = cols.sum(dim=1) / (2.0 * n)
    ok = (f > 0) & (f < 1)
    sd = torch.where(ok, torch.sqrt(2.0 * f * (1.0 - f)), torch.ones_like(f))
    X = torch.where(ok[:, None], (cols - 2.0 * f[:, None]) / sd[:, None], torch.zeros_like(cols))
    g = (X.T @ torch.as_tensor(b[pos], device=device)).cpu().numpy()
    vg = g.var()
    ve = vg * (1.0 - spec.h2) / spec.h2 if vg > 0 else 1.0
    y = spec.mean + g + rng.standard_normal(n) * np.sqrt(ve)
    return codes, y, b
