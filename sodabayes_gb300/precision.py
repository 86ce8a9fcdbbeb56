"""Error of a reduced-precision context against an FP64 context, stated on
one subset of one loaded state.

Both contexts hold the same genotypes, Z and chain states (loaded with
SodaJob.set_state) and the same iteration counter, so the counter-based draws
of every (chain, SNP) are the same uniforms in both.  For one subset this
measures:

  * the conditional right-hand sides x_j'r + u_j'ra (models.f90:154, 219,
    358) that each context's draw consumes, and the conditional means and
    standard deviations of the effect draw derived from them
    (models.f90:382-386), in units of the conditional standard deviation;
  * the class draws of BayesC/Cpi/R/Rc (models.f90:350-379): every (chain,
    SNP) whose class differs between the contexts is listed with its decision
    margin, the distance of its uniform from the nearest boundary of the
    FP64 cumulative class probabilities;
  * after the subset's residual update (models.f90:415-430), the residual
    identity yadj = y - mu - X g of each context, recomputed in FP64 here.

The uniform of a class draw is the first word of the Philox4x32-10 stream
keyed (seed, chain, iteration, SNP, purpose 1) that the kernels use; it is
recomputed here in numpy.  Used by the GPU tests and by bench.py.
"""
from __future__ import annotations

import numpy as np

from . import synth

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
_LO = np.uint64(0xFFFFFFFF)
P_SNP = 1


def philox_first_word(seed: int, chain, it: int, slot, purpose: int) -> np.ndarray:
    """First 64-bit output of the counter (it, slot, purpose, chain << 20)
    under key seed (Philox4x32-10, Salmon et al. 2011), vectorised over
    `slot` and `chain` (broadcast)."""
    slot = np.asarray(slot, dtype=np.uint32)
    chain = np.asarray(chain, dtype=np.uint32)
    shape = np.broadcast(slot, chain).shape
    c0 = np.full(shape, it, dtype=np.uint32)
    c1 = np.broadcast_to(slot, shape).astype(np.uint32)
    c2 = np.full(shape, purpose, dtype=np.uint32)
    c3 = (np.broadcast_to(chain, shape).astype(np.uint32) << np.uint32(20)).astype(np.uint32)
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    with np.errstate(over="ignore"):
        for r in range(10):
            if r:
                k0 = np.uint32(k0 + _W0)
                k1 = np.uint32(k1 + _W1)
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & _LO).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & _LO).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return (c1.astype(np.uint64) << np.uint64(32)) | c0.astype(np.uint64)


def class_uniform(seed: int, chain, it: int, snp, fp32: bool) -> np.ndarray:
    """The uniform of a class draw: FP64 draws map the word like
    rng_int64_to_real64 (parallelrng.f90:242-249); the FP32 draws of the
    reduced-precision modes take its top 24 bits, offset by half a unit."""
    w = philox_first_word(seed, chain, it, snp, P_SNP)
    if fp32:
        return ((w >> np.uint64(40)).astype(np.float64) + 0.5) * 2.0 ** -24
    return (w >> np.uint64(12)).astype(np.float64) * 2.0 ** -52


def class_cumulative(rhs_total, zz, vare, gp, log_p):
    """Cumulative class probabilities (models.f90:362-377) for right-hand
    sides that already include d*g: rows = SNPs, columns = classes 1..nm."""
    rhs = np.asarray(rhs_total, dtype=np.float64)
    nm = len(gp)
    s = np.empty(rhs.shape + (nm,))
    s[..., 0] = log_p[..., 0]
    for k in range(1, nm):
        logdet = np.log(gp[k] * zz / vare + 1.0)
        uhat = rhs / (zz + vare / gp[k])
        s[..., k] = -0.5 * (logdet - rhs * uhat / vare) + log_p[..., k]
    prob = np.empty_like(s)
    for k in range(nm):
        d = s - s[..., k:k + 1]
        d[..., k] = -np.inf
        over = np.any(d > 700, axis=-1)
        e = np.where(d < -700, 0.0, np.exp(np.minimum(d, 700)))
        prob[..., k] = np.where(over, 0.0, 1.0 / (1.0 + e.sum(axis=-1)))
    return np.cumsum(prob, axis=-1)


def sparse_state(G, y, spec_b, method_nmix, mix, vara, vare, incl, pi, groups, seed, naind):
    """A settled-looking chain state: a fraction `incl` of SNPs in non-zero
    classes with effects N(0, gamma_k vara), yadj = y - mu - X g in FP64,
    yAadj ~ N(0, vare).  Returns a dict for SodaJob.set_state."""
    rng = np.random.default_rng(seed)
    n, p = G.shape
    nm = method_nmix
    cls = np.ones(p, dtype=np.int32)
    g = np.zeros(p)
    nz = np.sort(rng.choice(p, size=max(1, int(incl * p)), replace=False))
    if nm == 2:
        cls[nz] = 2
    else:
        cls[nz] = rng.integers(2, nm + 1, size=len(nz))
    sd = np.sqrt(np.asarray(mix, dtype=np.float64)[cls[nz] - 1] * vara)
    g[nz] = rng.standard_normal(len(nz)) * sd
    mu = float(np.mean(y))
    r = y - mu - synth.centred(G[:, nz]) @ g[nz]
    ra = rng.standard_normal(naind) * np.sqrt(vare)
    return dict(g=g, cls=cls, vara_s=np.zeros(p), yadj=r, yaadj=ra, mu=mu, vare=vare, vara=vara,
                included=len(nz), pi=pi)


def conditional_check(job_lo, job_64, G, y, b: int, rep: int, states, groups=None, tau: float = 1e-4):
    """Runs subset b of iteration `rep` in both contexts from `states` (one
    dict per chain, for set_state) and returns the error statement (see the
    module docstring).  Class draws are compared for BayesC/Cpi/R/Rc."""
    cfg = job_64.cfg
    C = job_lo.chains
    for job in (job_lo, job_64):
        for c in range(C):
            job.set_state(c, **states[c])
        job.set_iteration(rep)
    rhs_lo = job_lo.subset_rhs(b)
    rhs_64 = job_64.subset_rhs(b)
    ls, le = job_64.subset_bounds(b)
    _, xxd, skip = job_64.z()
    zz = float(xxd[b])
    act = skip[ls:le] == 0
    scale = np.max(np.abs(rhs_64[:, act]))
    drhs = np.abs(rhs_lo - rhs_64)[:, act]
    out = {"subset": b, "snps": int(le - ls), "chains": C, "rhs_max_abs_err_over_max": float(drhs.max() / scale),
           "rhs_rms_rel": float(np.sqrt(np.mean(drhs ** 2)) / np.sqrt(np.mean(rhs_64[:, act] ** 2)))}
    # conditional mean and sd of the effect draw in each non-zero class, in units of that sd
    nm, ng = cfg.nmix, cfg.ngroup
    mix = np.array([cfg.mix[k] for k in range(nm)])
    snp = np.arange(ls, le)                       # identity order (no permvec)
    grp = (np.ones(len(snp), dtype=np.int64) if groups is None else np.asarray(groups)[snp]) - 1
    worst_mean = 0.0
    cls_total = cls_diff = 0
    margins = []
    fp32 = cfg.precision != 0
    for c in range(C):
        st = states[c]
        gp = mix * st["vara"]
        g_old = st["g"][snp]
        in_model = st["cls"][snp] > 1
        tot64 = rhs_64[c] + np.where(in_model, zz * g_old, 0.0)
        totlo = rhs_lo[c] + np.where(in_model, zz * g_old, 0.0)
        for k in range(1, nm):
            v1 = zz + st["vare"] / gp[k]
            sdk = np.sqrt(st["vare"] / v1)
            worst_mean = max(worst_mean, float(np.max(np.abs(totlo - tot64)[act] / v1 / sdk)))
        if cfg.method in (3, 4, 5, 6):
            pi = np.asarray(st["pi"], dtype=np.float64).reshape((ng, nm), order="F")
            cum = class_cumulative(tot64, zz, st["vare"], gp, np.log(pi[grp]))
            u = class_uniform(int(abs(cfg.seed)), c, rep, snp, fp32=False)
            margin = np.min(np.abs(u[:, None] - cum[:, :-1]), axis=1) if nm > 1 else np.full(len(snp), 1.0)
            margins.append(margin[act])
    for job in (job_lo, job_64):
        job.run_subset(b)
    res_err = 0.0
    for c in range(C):
        s_lo, s_64 = job_lo.state(c), job_64.state(c)
        if cfg.method in (3, 4, 5, 6):
            d = (s_lo["cls"][snp] != s_64["cls"][snp]) & act
            cls_total += int(act.sum())
            cls_diff += int(d.sum())
            for j in np.nonzero(d)[0]:
                out.setdefault("disagreements", []).append(
                    {"chain": c, "snp": int(snp[j]), "margin": float(margins[c][np.nonzero(act)[0].tolist().index(j)]),
                     "class_fp64": int(s_64["cls"][snp[j]]), "class_lo": int(s_lo["cls"][snp[j]])})
        if c in (0, C - 1):
            nz = np.nonzero(s_lo["g"])[0]
            r_host = y - s_lo["mu"] - (synth.centred(G[:, nz]) @ s_lo["g"][nz] if len(nz) else 0.0)
            res_err = max(res_err, float(np.max(np.abs(s_lo["yadj"] - r_host)) / np.max(np.abs(r_host))))
    out["cond_mean_max_err_in_sd"] = worst_mean
    out["residual_identity_rel_err"] = res_err
    if cls_total:
        allm = np.concatenate(margins)
        out["class_draws"] = cls_total
        out["class_disagreements"] = cls_diff
        out["tau"] = tau
        out["draws_with_margin_below_tau"] = int(np.sum(allm < tau))
        out["min_margin"] = float(allm.min())
        dis = out.get("disagreements", [])
        out["disagreements_above_tau"] = int(sum(1 for x in dis if x["margin"] >= tau))
        out["max_margin_of_a_disagreement"] = float(max((x["margin"] for x in dis), default=0.0))
    return out
