"""Benchmark of the SODA Gibbs step on the config-3 workload.

Workload: SODA BayesCpi, n=20,000 individuals, p=500,000 SNPs, subsets of
2,000 SNPs (250 subsets), genotypes from the seeded LD generator (50-SNP AR(1)
blocks, rho=0.7, maf~U(0.01,0.5)), 2,000 causal N(0,1) effects, h2=0.5.
A step is one Gibbs iteration of every chain.

Our arm (default): the batched FP8 sampler (16 chains on shared genotypes) is
the headline value, in Gibbs iterations x chains per second, device-timed with
inputs resident in HBM; the plain FP32 path (1 chain) is timed the same way,
and both are compared with an FP64 run of the same chain (same counter-based
draws) to state the error.  `e2e` runs the whole job through the C ABI from
host buffers (genotypes and phenotypes copied in, the .hyp trace and the
posterior means copied out) and divides its iterations x chains by the wall
time.  `cpu_baseline` times the CPU oracle (OpenMP, FP64) on a bounded sample.

--impl reference: the reference is Fortran and cannot be compiled here (no
Fortran compiler on either machine), so the reference arm times the CPU
restatement of its algorithm (oracle/) on the host cores.

Multi-GPU: the path does not shard (one chain's subsets are sequential);
--gpus N runs N independent replicas, one per rank.

--profile-case: a small case with the same per-subset shape (n=20,000,
p=20,000, 10 subsets of 2,000) for ncu captures of single kernel launches;
it runs --steps iterations and prints the library timings.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SODA Gibbs iters/s×chains, n=20k p=500k: batched FP8 vs plain FP32, same error"
UNIT = "iters*chains/s"
SPEC_KEY = "c3"
BLOCKSIZE = 2000
METHOD = "BayesCpi"


def _dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return rank, ws


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=float(np.median(sm)), sm_max_mhz=float(max(smax)), samples=len(sm),
                       power_w_max=float(max(power)) if power else None)
        out["reasons"] = sorted(reasons)
        return out


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# Priors on the scale of the simulated data: per-SNP effect variance ~1 (true
# effects N(0,1)) and residual variance ~2000 (var(y) ~ 4000 at h2 = 0.5).
PRIORS = dict(scale_va=1.0, df_va=4.0, scale_ve=2000.0, df_ve=4.0)


def _opts(prec, chains, seed, numit):
    from sodabayes_gb300 import JobOptions
    return JobOptions(method=METHOD, numit=numit, burnin=0, blocksize=BLOCKSIZE, seed=seed, precision=prec,
                      chains=chains, **PRIORS)


def _make_job(spec, codes_dev, y, prec, chains, seed, numit=100000):
    from sodabayes_gb300 import SodaJob, make_config
    job = SodaJob(make_config(spec.n, spec.p, _opts(prec, chains, seed, numit)))
    job.load_genotypes(device_ptr=codes_dev.data_ptr())
    job.load_pheno(y)
    job.build_z()
    job.init_chains()
    return job


def _rhs_bytes(n, N, chains, prec, tc=False):
    """Algorithmic bytes of one rhs launch: the subset's genotype columns and
    augmenting columns once, plus each chain's residual copies.  The
    tensor-core rhs reads the genotype codes 2-bit packed (n N / 4 bytes), the
    upper triangle of U as three bf16 terms and the residuals r and ra as their
    three-term bf16 splits."""
    if tc:
        return n * N // 4 + N * (N + 1) // 2 * 6 + chains * (n + N) * 6
    ex = {"fp8": 1, "fp32": 4, "fp64": 1}[prec]
    eu = {"fp8": 4, "fp32": 4, "fp64": 8}[prec]
    er = {"fp8": 4, "fp32": 4, "fp64": 8}[prec]
    return n * N * ex + N * (N + 1) // 2 * eu + chains * (n * er + N * 8)


def _update_bytes(n, N, chains):
    """Algorithmic bytes of one tensor-core update launch (every stage
    active): the subset's genotype codes 2-bit packed (n N / 4 bytes) and the
    three bf16 terms of the upper triangle of U once, the delta split once,
    and each chain's FP64 residual read and written with its bf16 split."""
    return n * N // 4 + N * (N + 1) // 2 * 6 + 3 * chains * N * 2 + chains * n * (8 + 8 + 6)


def bench_ours(args, rank, ws):
    import torch

    import ctypes

    from sodabayes_gb300 import SodaJob, _abi, make_config, synth
    spec = synth.CONFIGS[SPEC_KEY]
    spec = synth.SynthSpec(**{**spec.__dict__, "seed": spec.seed + 1000 * rank})
    codes, y, _ = synth.make_device(spec)
    torch.cuda.synchronize()
    C = args.chains
    K, W = args.steps, args.warmup
    res = {}

    # ---- headline: batched FP8, inputs resident -----------------------------------
    job = _make_job(spec, codes, y, "fp8", C, 77 + rank)
    job.run(args.settle + W)
    _barrier(ws)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        job.run(K)
        torch.cuda.synchronize()
    _barrier(ws)
    dev_ms = job.timings()[2]
    st = job.state(0)
    prof = job.profile_kernels(2)
    job.close()
    t_max = _max_over_ranks(dev_ms, ws)
    units = _sum_over_ranks(float(K * C), ws)
    res["value"] = units / (t_max / 1000.0)
    res["ms_per_step"] = t_max / K
    res["clocks"] = clk.summary()
    res["included_at_timing"] = st["included"]
    nb = spec.p // BLOCKSIZE
    hbm, peak_kind = _peaks()
    kms = {k: round(v[0] / 2, 4) for k, v in prof.items()}

    def _roof(cls, kernel, nbytes):
        ms = prof[cls][0] / prof[cls][1]
        achieved = nbytes / (ms / 1000.0) / 1e9
        return {"bound": "hbm", "kernel": kernel % C, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4),
                "traffic": _measured_traffic(kernel.split("<")[0] + "%d_n20000_s2000.md" % C),
                "traffic_source": "ncu --set full of one launch of the same kernel at the same subset shape "
                                  "(profiles/%s%d_n20000_s2000.md)" % (kernel.split("<")[0], C),
                "peak_source": peak_kind, "bytes_per_launch": nbytes, "launch_ms": round(ms, 5)}

    # the dominant kernel (the residual update), then the rhs
    res["roofline"] = _roof("update", "k_update_tc<%d>", _update_bytes(spec.n, BLOCKSIZE, C))
    res["roofline"]["kernel_ms_per_iter"] = kms
    res["roofline_rhs"] = _roof("rhs", "k_rhs_tc<%d>", _rhs_bytes(spec.n, BLOCKSIZE, C, "fp8", tc=True))
    res["gpu_launches"] = K * (3 + 3 * nb + 5)   # mu; rhs, draws, update per subset; hyper/stats/recal

    # ---- plain FP32 path (1 chain), same timing -----------------------------------
    job = _make_job(spec, codes, y, "fp32", 1, 77 + rank)
    job.run(args.settle + W)
    torch.cuda.synchronize()
    job.run(K)
    fp32_ms = job.timings()[2]
    job.close()
    res["fp32_plain"] = {"value": K / (fp32_ms / 1000.0), "ms_per_step": fp32_ms / K, "chains": 1}

    # ---- error against FP64 runs of the same chains ---------------------------------
    # The headline's own kernels: the FP8 context with the headline's chain count runs on the
    # tensor cores (k_rhs_tc / k_draw / k_update_tc); chains 0 and 1 are compared with an FP64
    # context of two chains (same seed: every draw uses the same counter-based uniforms).
    res["error_vs_fp64"] = error_vs_fp64(spec, codes, y, C, args.error_iters)
    res["conditional_check"] = conditional_check_c3(codes, y, C)
    if args.accept_iters > 0:
        res["acceptance"] = acceptance(spec, codes, y, C, args.accept_burnin, args.accept_iters)

    # ---- e2e: the whole job through the C ABI, host buffers in and out ------------
    host_codes = torch.empty(codes.shape, dtype=torch.int8, pin_memory=True)
    host_codes.copy_(codes)
    del codes
    torch.cuda.empty_cache()
    Ke = args.e2e_steps
    rows = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    job = SodaJob(make_config(spec.n, spec.p, _opts("fp8", C, 77 + rank, Ke)))
    job.load_genotypes(host_ptr=host_codes.data_ptr())
    job.load_pheno(y)
    t_up = time.perf_counter()
    job.build_z()
    job.init_chains()
    t_setup = time.perf_counter()
    job.run(Ke, trace=lambda r: rows.append(r.rep))
    t_run = time.perf_counter()
    outs = [job.results(c) for c in range(C)]
    job.close()
    t_e2e = time.perf_counter() - t0
    phases = {"create_and_upload_s": round(t_up - t0, 3), "z_build_and_init_s": round(t_setup - t_up, 3),
              "iterations_s": round(t_run - t_setup, 3), "results_s": round(t0 + t_e2e - t_run, 3)}
    t_e2e = _max_over_ranks(t_e2e, ws)
    units_e2e = _sum_over_ranks(float(Ke * C), ws)
    h2d = spec.n * spec.p + 8 * spec.n
    d2h = len(rows) * ctypes.sizeof(_abi.TraceRow) + C * 8 * spec.p * 5
    res["e2e"] = {"value": units_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d / Ke),
                  "d2h_bytes_per_step": int(d2h / Ke), "iterations": Ke, "wall_s": round(t_e2e, 3),
                  "includes": "create, genotype+phenotype upload, Z build, init, iterations with .hyp trace, "
                              "posterior means download", "phases": phases}
    del outs
    return res


def _err(a, b):
    d = a["g"] - b["g"]
    return {"g_rel_rms": float(np.sqrt(np.mean(d ** 2)) / max(1e-300, np.sqrt(np.mean(b["g"] ** 2)))),
            "class_agreement": float(np.mean(a["cls"] == b["cls"])),
            "vare_rel": float(abs(a["vare"] / b["vare"] - 1))}


def error_vs_fp64(spec, codes, y, C, E):
    """State after E iterations of the FP8 context with C chains (tensor-core kernels when C is 4, 8
    or 16) and of the plain FP32 context (1 chain) against FP64 contexts of the same seed."""
    st = {}
    for prec, chains in (("fp64", 2), ("fp8", C), ("fp32", 1)):
        job = _make_job(spec, codes, y, prec, chains, 99)
        job.run(E)
        st[prec] = [job.state(c) for c in range(min(chains, 2))]
        job.close()
    out = {"iterations": E,
           "fp8": {"kernels": "k_rhs_tc<%d>, k_draw<fp8,%d,tc>, k_update_tc<%d> (the headline's)" % (C, C, C)
                   if C in (4, 8, 16) else "k_rhs<fp8,%d>, k_draw, k_update<fp8,%d>" % (C, C),
                   "chains_compared": [0, 1]},
           "fp32": {"kernels": "k_rhs<fp32,1>, k_draw<fp32,1>, k_update<fp32,1> (the plain FP32 path)",
                    "chains_compared": [0]}}
    for c in range(min(C, 2)):
        out["fp8"]["chain%d" % c] = _err(st["fp8"][c], st["fp64"][c])
    out["fp32"]["chain0"] = _err(st["fp32"][0], st["fp64"][0])
    out["nonzero_effects_fp64"] = int(np.sum(st["fp64"][0]["g"] != 0))
    return out


def conditional_check_c3(codes, y, C, nsub=2):
    """One subset of one loaded state (a settled-looking sparse state, 1% of SNPs in the model) at the
    config-3 subset shape, FP8 with C chains against FP64 with C chains: right-hand sides, conditional
    means, class draws with their decision margins, residual identity after the update.  The first
    nsub subsets of the workload's genotypes (n = 20,000) serve as the data."""
    from sodabayes_gb300 import precision
    G = np.asfortranarray(codes[:nsub * BLOCKSIZE].cpu().numpy().T)
    jobs = {}
    for prec in ("fp8", "fp64"):
        from sodabayes_gb300 import JobOptions, SodaJob, make_config
        cfg = make_config(G.shape[0], G.shape[1], JobOptions(method=METHOD, numit=100, burnin=0,
                                                             blocksize=BLOCKSIZE, seed=4242, precision=prec,
                                                             chains=C, **PRIORS))
        job = SodaJob(cfg)
        job.load_genotypes(G)
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        jobs[prec] = job
    vare = 0.5 * float(np.var(y))
    states = [precision.sparse_state(G, y, None, 2, (0.0, 1.0), 1.0, vare, 0.01, np.array([[0.99, 0.01]]), None,
                                     seed=1000 + c, naind=BLOCKSIZE) for c in range(C)]
    try:
        res = precision.conditional_check(jobs["fp8"], jobs["fp64"], G, y, 0, 7, states, tau=1e-4)
    finally:
        for j in jobs.values():
            j.close()
    res["shape"] = "n=%d, subset %d, %d chains, BayesCpi" % (G.shape[0], BLOCKSIZE, C)
    dis = res.pop("disagreements", [])
    res["disagreement_margins"] = [round(x["margin"], 9) for x in dis][:20]
    return res


def _batch_means(x):
    """(mean, Monte-Carlo standard error, effective sample size) of a trace by
    non-overlapping batch means with batches of floor(sqrt(N))."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    b = max(1, int(np.sqrt(n)))
    nb = n // b
    bm = x[:nb * b].reshape(nb, b).mean(axis=1)
    var_bm = b * bm.var(ddof=1) if nb > 1 else 0.0
    se = float(np.sqrt(var_bm / n)) if var_bm > 0 else 0.0
    v = x.var(ddof=1)
    ess = float(n * v / var_bm) if var_bm > 0 else float(n)
    return float(x.mean()), se, min(ess, float(n))


def acceptance(spec, codes, y, C, burn, keep):
    """Free-running chains of the n=20000, p=500000 workload (acceptance): the FP8 sampler with C chains, the plain
    FP32 path (1 chain) and two FP64 runs (1 chain each, seeds A and B: the Monte-Carlo floor of two
    independent FP64 runs).  Posterior means of the SNP effects and GEBVs (compute_dgv,
    utilities.f90:616-622, of the posterior means, models.f90:576-598), pi = included / p, the model's
    genetic variance share h2 = sum_k n_k gamma_k s2g / (that + s2e) and s2e per kept iteration with
    batch-means standard errors, and effective samples per second of mu, s2e and s2g."""
    seeds = {"fp64": 77, "fp64_seedB": 78, "fp8": 77, "fp32": 77}
    runs = {}
    for name, prec, chains in (("fp64", "fp64", 1), ("fp64_seedB", "fp64", 1), ("fp8", "fp8", C),
                               ("fp32", "fp32", 1)):
        from sodabayes_gb300 import JobOptions, SodaJob, make_config
        opts = JobOptions(method=METHOD, numit=burn + keep, burnin=burn, blocksize=BLOCKSIZE, seed=seeds[name],
                          precision=prec, chains=chains, **PRIORS)
        job = SodaJob(make_config(spec.n, spec.p, opts))
        job.load_genotypes(device_ptr=codes.data_ptr())
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        job.run(burn)
        rows = []
        job.run(keep, trace=lambda r: rows.append((r.chain, r.mu, r.vare, r.vara, r.included)))
        dev_s = job.timings()[2] / 1000.0
        res = [job.results(c) for c in range(chains)]
        gebv = [job.compute_dgv(r["mu_store"], r["gstore"]) for r in res[:2]]
        avg = np.mean([r["gstore"] for r in res], axis=0)
        mu_avg = float(np.mean([r["mu_store"] for r in res]))
        gebv_avg = job.compute_dgv(mu_avg, avg) if chains > 1 else gebv[0]
        job.close()
        tr = np.array(rows)
        per = {}
        ess = {"mu": 0.0, "vare": 0.0, "vara": 0.0}
        for c in range(chains):
            t = tr[tr[:, 0] == c]
            for k, col in (("mu", 1), ("vare", 2), ("vara", 3)):
                ess[k] += _batch_means(t[:, col])[2]
            vg = t[:, 3] * t[:, 4]                   # BayesCpi: included SNPs x effect variance
            per[c] = {"pi": _batch_means(t[:, 4] / spec.p), "h2": _batch_means(vg / (vg + t[:, 2])),
                      "vare": _batch_means(t[:, 2])}
        runs[name] = {"g": [r["gstore"] for r in res[:2]], "g_avg": avg, "gebv": gebv, "gebv_avg": gebv_avg,
                      "per": per, "ess_per_s": {k: v / dev_s for k, v in ess.items()}, "device_s": dev_s,
                      "chains": chains}

    def rel_rms(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))

    ref = runs["fp64"]
    out = {"burn_in": burn, "kept": keep, "seeds": seeds,
           "targets": {"effects_rel_rms_max": 1e-3, "gebv_corr_min": 0.9999, "pi_h2_vare_within_z": 3.0}}
    for name in ("fp8", "fp32", "fp64_seedB"):
        r = runs[name]
        e = {"effects_rel_rms_chain0": rel_rms(r["g"][0], ref["g"][0]),
             "gebv_corr_chain0": float(np.corrcoef(r["gebv"][0], ref["gebv"][0])[0, 1])}
        if r["chains"] > 1:
            e["effects_rel_rms_mean_of_chains"] = rel_rms(r["g_avg"], ref["g"][0])
            e["gebv_corr_mean_of_chains"] = float(np.corrcoef(r["gebv_avg"], ref["gebv"][0])[0, 1])
        z = {}
        for k in ("pi", "h2", "vare"):
            m, se = r["per"][0][k][0], r["per"][0][k][1]
            m0, se0 = ref["per"][0][k][0], ref["per"][0][k][1]
            z[k] = {"mean": m, "se": se, "fp64_mean": m0, "fp64_se": se0,
                    "z": float(abs(m - m0) / max(1e-300, np.sqrt(se * se + se0 * se0)))}
        e["chain0_vs_fp64"] = z
        e["pass"] = {"effects": e["effects_rel_rms_chain0"] <= 1e-3, "gebv": e["gebv_corr_chain0"] >= 0.9999,
                     "pi_h2_vare": all(v["z"] <= 3.0 for v in z.values())}
        e["ess_per_s"] = r["ess_per_s"]
        e["chains"] = r["chains"]
        out[name] = e
    out["fp64"] = {"ess_per_s": ref["ess_per_s"], "chains": 1}
    out["note"] = ("fp64_seedB is a second FP64 chain with another seed: its distance from the FP64 run is the "
                   "Monte-Carlo floor of the comparison.  Same-seed chains share every uniform, so their "
                   "trajectories coincide until the first class decision whose margin is below the FP32 "
                   "rounding of the draw; after that they differ by Monte-Carlo error.")
    return out


def cpu_sample(args, steps=1, warmup=0):
    """The CPU oracle (FP64, OpenMP over the host cores) on a bounded sample of
    the same workload: NB_SAMPLE of the 250 subsets of one iteration at full n,
    in the sparse state of a settled chain; iterations/s are extrapolated
    linearly in subsets."""
    import torch

    from oracle import oracle as O
    from sodabayes_gb300 import make_config, synth
    spec = synth.CONFIGS[SPEC_KEY]
    nbs = args.cpu_blocks
    ps = nbs * BLOCKSIZE
    sspec = synth.SynthSpec(**{**spec.__dict__, "p": ps, "ncausal": max(1, spec.ncausal * ps // spec.p)})
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    codes, y, _ = synth.make_device(sspec, device=dev)
    G = codes.cpu().numpy().T        # (n, ps) column-major view
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o = O.Oracle(make_config(sspec.n, ps, _opts("fp64", 1, 77, 100000)))
    o.load_genotypes(G)
    o.load_pheno(y)
    o.build_z(power_maxit=-1)      # Gershgorin d: the setup is not timed
    o.init_chains()
    o.set_sparse_state(0.01, 5)
    for _ in range(warmup):
        o.run_blocks(0, nbs, 1)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.run_blocks(0, nbs, 1)
        times.append(time.perf_counter() - t0)
    o.close()
    per_block = float(np.median(times)) / nbs
    t_iter = per_block * (spec.p // BLOCKSIZE)
    return {"value": 1.0 / t_iter, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{nbs} of {spec.p // BLOCKSIZE} subsets (n={spec.n}, {ps} SNPs) of one BayesCpi iteration "
                      f"in the sparse state of a settled chain (1% of SNPs in the model), FP64, {cores} OpenMP "
                      f"threads; iterations/s extrapolated linearly in subsets; median of {steps}",
            "seconds_per_iteration": t_iter}


def workload_c5(args):
    """Config 5 on one GPU: BayesRc, 16 chains on shared genotypes, three annotation classes (0.1, 0.3, 0.6),
    4-class mixtures, n=50,000, p=1,000,000, subset 1000.  Prints its own JSON line: iterations x chains / s
    of the batched FP8 sampler (inputs resident, CUDA-event timed) and the error of one chain against an FP64
    run of the same chain.  The default run (config 3) is unchanged."""
    import torch
    from sodabayes_gb300 import JobOptions, SodaJob, make_config, synth
    spec = synth.CONFIGS["c5"]
    groups = synth.annotation_groups(spec.p)
    t0 = time.perf_counter()
    codes, y, _ = synth.make_device(spec)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    vy = float(np.var(y))

    def job_of(prec, chains, seed):
        o = JobOptions(method="BayesRc", nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2), ngroup=3, numit=100000, burnin=0,
                       blocksize=1000, seed=seed, precision=prec, chains=chains, scale_va=0.5 * vy, df_va=4.0,
                       scale_ve=0.5 * vy, df_ve=4.0)
        job = SodaJob(make_config(spec.n, spec.p, o))
        job.load_genotypes(device_ptr=codes.data_ptr())
        job.load_pheno(y)
        job.set_groups(groups)
        t = time.perf_counter()
        job.build_z()
        job.init_chains()
        torch.cuda.synchronize()
        return job, time.perf_counter() - t

    C, K = args.chains, args.steps
    job, t_setup = job_of("fp8", C, 77)
    job.run(args.settle + args.warmup)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        job.run(K)
        torch.cuda.synchronize()
    dev_ms = job.timings()[2]
    free, total = torch.cuda.mem_get_info()
    used_gb = (total - free) / 1e9
    job.close()
    E = args.error_iters
    st = {}
    for prec, chains in (("fp64", 2), ("fp8", C)):
        job, _ = job_of(prec, chains, 99)
        job.run(E)
        st[prec] = [job.state(c) for c in range(2)]
        job.close()
    err = {"iterations": E, "kernels": "k_rhs_tc<%d>, k_draw<fp8,%d,tc>, k_update_tc<%d>" % (C, C, C),
           "chain0": _err(st["fp8"][0], st["fp64"][0]), "chain1": _err(st["fp8"][1], st["fp64"][1])}
    # one subset of one loaded state at the config-5 subset shape (n = 50,000, subsets of 1,000, BayesRc in
    # three groups): the first two subsets of the workload's genotypes
    from sodabayes_gb300 import precision
    G = np.asfortranarray(codes[:2000].cpu().numpy().T)
    del codes
    torch.cuda.empty_cache()
    g2 = groups[:2000]
    jobs = {}
    for prec in ("fp8", "fp64"):
        o = JobOptions(method="BayesRc", nmix=4, mix=(0.0, 1e-4, 1e-3, 1e-2), ngroup=3, numit=100, burnin=0,
                       blocksize=1000, seed=4242, precision=prec, chains=C, scale_va=0.5 * vy, df_va=4.0,
                       scale_ve=0.5 * vy, df_ve=4.0)
        j = SodaJob(make_config(G.shape[0], G.shape[1], o))
        j.load_genotypes(G)
        j.load_pheno(y)
        j.set_groups(g2)
        j.build_z()
        j.init_chains()
        jobs[prec] = j
    pi = np.array([[0.97, 0.015, 0.01, 0.005], [0.95, 0.03, 0.015, 0.005], [0.99, 0.006, 0.003, 0.001]])
    states = [precision.sparse_state(G, y, None, 4, (0.0, 1e-4, 1e-3, 1e-2), 1.0, 0.5 * vy, 0.01, pi, g2,
                                     seed=1000 + c, naind=1000) for c in range(C)]
    try:
        cond = precision.conditional_check(jobs["fp8"], jobs["fp64"], G, y, 0, 7, states, groups=g2, tau=1e-4)
    finally:
        for j in jobs.values():
            j.close()
    dis = cond.pop("disagreements", [])
    cond["disagreement_margins"] = [round(x["margin"], 9) for x in dis][:20]
    cond["shape"] = "n=50000, subset 1000, %d chains, BayesRc (3 groups, 4 classes)" % C
    line = {"workload": "config 5: SODA BayesRc n=50000 p=1000000 subset 1000 (1000 subsets), 16 chains on shared "
                        "genotypes, 3 annotation classes (0.1, 0.3, 0.6), mixture (0, 1e-4, 1e-3, 1e-2), LD generator "
                        "(100-SNP AR(1) blocks rho=0.8, maf~U(0.01,0.5)), 5000 causal effects, h2=0.5",
            "metric": "SODA Gibbs iters/s x chains", "value": K * C / (dev_ms / 1000.0), "unit": UNIT,
            "ms_per_step": dev_ms / K, "chains": C, "steps": K, "warmup": args.warmup,
            "settle_iterations": args.settle, "precision": "fp8", "data": "synthetic (seeded generator of config 5)",
            "error_vs_fp64": err, "conditional_check": cond,
            "device_gb_in_use_fp8_job": round(used_gb, 1), "generate_s": round(t_gen, 2),
            "z_build_and_init_s": round(t_setup, 2), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def workload_c4(args):
    """Config 4 on one GPU: 32 independent BayesB analyses, n ~ U[500, 20000], p ~ U[10000, 200000], LD
    generator of config 2, h2 ~ U(0.1, 0.7), 0.5% of p causal, FP8, one chain each, subset sizes from the batch
    autotuner, all analyses in one launch per kernel under one captured CUDA graph (SodaBatch).  Prints its own
    JSON line: analysis iterations per second of the batch (CUDA-event timed, inputs resident), beside the same
    analyses run one after another, each under its own graph, and the autotuner's modelled time."""
    import torch
    from sodabayes_gb300 import JobOptions, SodaBatch, SodaJob, autotune_batch, make_config, synth
    J = 32
    rng = np.random.default_rng(20260004)
    n = rng.integers(500, 20001, size=J)
    p = rng.integers(10000, 200001, size=J)
    h2 = rng.uniform(0.1, 0.7, size=J)
    t0 = time.perf_counter()
    bs, steps, model_s = autotune_batch(n, p, 2000, max_blocksize=2000)
    t_tune = time.perf_counter() - t0
    jobs, t_gen, t_setup = [], 0.0, 0.0
    for j in range(J):
        spec = synth.SynthSpec(n=int(n[j]), p=int(p[j]), maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7,
                               ncausal=max(1, int(round(0.005 * p[j]))), h2=float(h2[j]), seed=20264000 + j)
        t = time.perf_counter()
        codes, y, _ = synth.make_device(spec)
        torch.cuda.synchronize()
        t_gen += time.perf_counter() - t
        vy = float(np.var(y))
        o = JobOptions(method="BayesB", blocksize=int(bs[j]), numit=2000, burnin=0, seed=91 + j, precision="fp8",
                       chains=1, kernels="cuda_cores", scale_va=0.5 * vy, df_va=4.0, scale_ve=0.5 * vy, df_ve=4.0)
        t = time.perf_counter()
        job = SodaJob(make_config(spec.n, spec.p, o))
        job.load_genotypes(device_ptr=codes.data_ptr())
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        torch.cuda.synchronize()
        t_setup += time.perf_counter() - t
        del codes
        jobs.append(job)
    torch.cuda.empty_cache()
    free, total = torch.cuda.mem_get_info()
    K, W = args.steps, args.warmup
    batch = SodaBatch(jobs)
    batch.run(args.settle + W)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        batch.run(K)
        torch.cuda.synchronize()
    ms, nsteps = batch.timings()
    batch.close()
    # the same analyses one after another, each under its own graph
    alone_ms = 0.0
    for job in jobs:
        job.run(W)
        job.run(K)
        alone_ms += job.timings()[2]
    for job in jobs:
        job.close()
    modelled_iter_s = (model_s - sum(
        int(p[j]) * (int(n[j]) * int(bs[j]) / 5e13 + int(bs[j]) ** 2 / (3 * 6e11)) for j in range(J))) / 2000
    line = {"workload": "config 4: 32 independent SODA BayesB analyses in one launch per kernel, n~U[500,20000], "
                        "p~U[10000,200000], LD generator of config 2 (50-SNP AR(1) blocks rho=0.7, maf~U(0.01,0.5)), "
                        "h2~U(0.1,0.7), 0.5% of p causal, FP8, 1 chain each, subset sizes autotuned",
            "metric": "SODA Gibbs analysis iterations/s (iterations x analyses)", "value": K * J / (ms / 1000.0),
            "unit": "iters*analyses/s", "ms_per_step": ms / K, "steps": K, "warmup": W,
            "settle_iterations": args.settle, "precision": "fp8", "kernels": "CUDA cores (one chain per analysis)",
            "data": "synthetic (seeded generator of config 2 per analysis)",
            "one_by_one": {"value": K * J / (alone_ms / 1000.0), "ms_per_step": alone_ms / K,
                           "how": "the same 32 jobs, each run on its own stream and graph, one after another"},
            "speedup_vs_one_by_one": alone_ms / ms,
            "launches_per_iteration": 3 + 3 * nsteps + 6, "subset_steps": nsteps,
            "autotune": {"blocksizes": [int(x) for x in bs], "steps": steps, "modelled_iteration_ms":
                         round(1000 * modelled_iter_s, 3), "measured_iteration_ms": round(ms / K, 3),
                         "tune_s": round(t_tune, 4)},
            "n": [int(x) for x in n], "p": [int(x) for x in p], "genotype_bytes": int(np.sum(n * p)),
            "device_gb_in_use": round((total - free) / 1e9, 1), "generate_s": round(t_gen, 1),
            "z_build_and_init_s": round(t_setup, 1), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def profile_case(args):
    """Small case for kernel captures: same per-subset shape as the workload."""
    import torch
    from sodabayes_gb300 import SodaJob, make_config, synth
    spec = synth.SynthSpec(n=20000, p=20000, maf_lo=0.01, maf_hi=0.5, ld_block=50, rho=0.7, ncausal=80, h2=0.5,
                           seed=5)
    codes, y, _ = synth.make_device(spec)
    with SodaJob(make_config(spec.n, spec.p, _opts(args.precision, args.chains, 77, 1000))) as job:
        job.load_genotypes(device_ptr=codes.data_ptr())
        job.load_pheno(y)
        job.build_z()
        job.init_chains()
        job.run(args.steps)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": {"n": spec.n, "p": spec.p, "chains": args.chains,
                                            "precision": args.precision, "iterations": args.steps,
                                            "included": job.state()["included"], "timings": job.timings()}}))


def _measured_traffic(kernel_file: str):
    """dram bytes read + written per launch from a committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", kernel_file)
    try:
        txt = open(path).read()
    except OSError:
        return None
    vals = {}
    for key in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
        for line in txt.splitlines():
            if line.startswith("| " + key + " |"):
                tok = line.split("|")[2].split()
                vals[key] = float(tok[0]) * {"MB": 1e6, "KB": 1e3, "GB": 1e9}.get(tok[1], 1.0)
    if len(vals) != 2:
        return None
    return vals["dram__bytes_read.sum"] + vals["dram__bytes_write.sum"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chains", type=int, default=16)
    ap.add_argument("--settle", type=int, default=60, help="untimed iterations before the warm-up")
    ap.add_argument("--error-iters", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--accept-iters", type=int, default=500,
                    help="kept iterations of the free-running acceptance comparison (0 skips it)")
    ap.add_argument("--accept-burnin", type=int, default=100)
    ap.add_argument("--cpu-blocks", type=int, default=4)
    ap.add_argument("--profile-case", action="store_true",
                    help="n=20000, p=20000 case of the same subset shape, for ncu captures")
    ap.add_argument("--precision", default="fp8", choices=["fp64", "fp32", "fp8"], help="--profile-case only")
    ap.add_argument("--workload", default="c3", choices=["c3", "c4", "c5"],
                    help="c4: config 4 (32 BayesB analyses in one launch per kernel); c5: config 5 (BayesRc, "
                         "n=50000, p=1000000, 16 chains); each on its own JSON line")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one replica per GPU: relaunch this command under torch.distributed.run
        import socket
        with socket.socket() as so:
            so.bind(("127.0.0.1", 0))
            port = so.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
               "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
        os.execv(sys.executable, cmd)
    if args.profile_case:
        profile_case(args)
        return
    if args.workload == "c4":
        if args.warmup < 3:
            args.warmup = 3
        workload_c4(args)
        return
    if args.workload == "c5":
        if args.warmup < 3:
            args.warmup = 3
        workload_c5(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    rank, ws = _dist_init()
    config = {"workload": "config 3: SODA BayesCpi n=20000 p=500000 subset 2000 (250 subsets), LD generator "
                          "(50-SNP AR(1) blocks rho=0.7, maf~U(0.01,0.5)), 2000 causal effects, h2=0.5",
              "n": 20000, "p": 500000, "blocksize": BLOCKSIZE, "method": METHOD, "priors": PRIORS,
              "l2_policy": "inputs larger than L2 (10 GB of genotype codes per iteration vs 126 MB L2)"}
    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_sample(args, steps=args.steps, warmup=min(args.warmup, 1))
        line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / cb["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator of config 3)", "config": {**config, "chains": 1},
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference is Fortran; no Fortran compiler exists on this machine or the GPU box, so "
                        "its algorithm runs as the CPU restatement in oracle/ (FP64, OpenMP)"}
        print(json.dumps(line), flush=True)
        return
    res = bench_ours(args, rank, ws)
    if rank == 0:
        cb = cpu_sample(args, steps=3, warmup=1)
        line = {"metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "2-bit packed genotype codes widened to exact bf16 0/1/2 on chip x bf16 hi/mid/lo splits "
                         "of the residuals, delta and U; FP32 accumulation, FP32 draws, FP64 residual masters",
                "data": "synthetic (seeded generator of config 3)",
                "config": {**config, "chains": args.chains, "precision": "fp8", "settle_iterations": args.settle,
                           "parallelism": f"replicas x{ws}"},
                "fp32_plain": res["fp32_plain"],
                "speedup_vs_fp32_plain": res["value"] / ws / res["fp32_plain"]["value"],
                "error_vs_fp64": res["error_vs_fp64"], "conditional_check": res["conditional_check"],
                "acceptance": res.get("acceptance"),
                "roofline": res["roofline"], "roofline_rhs": res["roofline_rhs"],
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
                "included_at_timing": res["included_at_timing"]}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
