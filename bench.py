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
    tensor-core rhs reads the upper triangle of U as three bf16 terms and the
    residuals r and ra as their three-term bf16 splits."""
    if tc:
        return n * N + N * (N + 1) // 2 * 6 + chains * (n + N) * 6
    ex = {"fp8": 1, "fp32": 4, "fp64": 1}[prec]
    eu = {"fp8": 4, "fp32": 4, "fp64": 8}[prec]
    er = {"fp8": 4, "fp32": 4, "fp64": 8}[prec]
    return n * N * ex + N * (N + 1) // 2 * eu + chains * (n * er + N * 8)


def _update_bytes(n, N, chains):
    """Algorithmic bytes of one tensor-core update launch (every stage
    active): the subset's genotype columns and the three bf16 terms of the
    upper triangle of U once, the delta split once, and each chain's FP64
    residual read and written with its bf16 split."""
    return n * N + N * (N + 1) // 2 * 6 + 3 * chains * N * 2 + chains * n * (8 + 8 + 6)


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

    # ---- error against an FP64 run of the same chain ------------------------------
    E = args.error_iters
    g = {}
    for prec in ("fp64", "fp32", "fp8"):
        job = _make_job(spec, codes, y, prec, 1, 99)
        job.run(E)
        s = job.state(0)
        g[prec] = (s["g"], s["cls"], s["mu"], s["vare"])
        job.close()
    err = {}
    for prec in ("fp32", "fp8"):
        d = g[prec][0] - g["fp64"][0]
        nz = g["fp64"][0] != 0
        err[prec] = {"g_rel_rms": float(np.sqrt(np.mean(d ** 2)) / max(1e-300, np.sqrt(np.mean(g["fp64"][0] ** 2)))),
                     "class_agreement": float(np.mean(g[prec][1] == g["fp64"][1])),
                     "vare_rel": float(abs(g[prec][3] / g["fp64"][3] - 1)),
                     "nonzero_effects_fp64": int(nz.sum())}
    res["error_vs_fp64"] = {"iterations": E, **err}

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
    job.build_z()
    job.init_chains()
    job.run(Ke, trace=lambda r: rows.append(r.rep))
    outs = [job.results(c) for c in range(C)]
    job.close()
    t_e2e = time.perf_counter() - t0
    t_e2e = _max_over_ranks(t_e2e, ws)
    units_e2e = _sum_over_ranks(float(Ke * C), ws)
    h2d = spec.n * spec.p + 8 * spec.n
    d2h = len(rows) * ctypes.sizeof(_abi.TraceRow) + C * 8 * spec.p * 5
    res["e2e"] = {"value": units_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d / Ke),
                  "d2h_bytes_per_step": int(d2h / Ke), "iterations": Ke, "wall_s": round(t_e2e, 3),
                  "includes": "create, genotype+phenotype upload, Z build, init, iterations with .hyp trace, "
                              "posterior means download"}
    del outs
    return res


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
    g = {}
    for prec in ("fp64", "fp8"):
        job, _ = job_of(prec, 1, 99)
        job.run(E)
        st = job.state(0)
        g[prec] = (st["g"], st["cls"], st["vare"])
        job.close()
    d = g["fp8"][0] - g["fp64"][0]
    line = {"workload": "config 5: SODA BayesRc n=50000 p=1000000 subset 1000 (1000 subsets), 16 chains on shared "
                        "genotypes, 3 annotation classes (0.1, 0.3, 0.6), mixture (0, 1e-4, 1e-3, 1e-2), LD generator "
                        "(100-SNP AR(1) blocks rho=0.8, maf~U(0.01,0.5)), 5000 causal effects, h2=0.5",
            "metric": "SODA Gibbs iters/s x chains", "value": K * C / (dev_ms / 1000.0), "unit": UNIT,
            "ms_per_step": dev_ms / K, "chains": C, "steps": K, "warmup": args.warmup,
            "settle_iterations": args.settle, "precision": "fp8", "data": "synthetic (seeded generator of config 5)",
            "error_vs_fp64": {"iterations": E, "g_rel_rms": float(np.sqrt(np.mean(d ** 2)) /
                                                                  max(1e-300, np.sqrt(np.mean(g["fp64"][0] ** 2)))),
                              "class_agreement": float(np.mean(g["fp8"][1] == g["fp64"][1])),
                              "vare_rel": float(abs(g["fp8"][2] / g["fp64"][2] - 1))},
            "device_gb_in_use_fp8_job": round(used_gb, 1), "generate_s": round(t_gen, 2),
            "z_build_and_init_s": round(t_setup, 2), "clocks": clk.summary()}
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
    ap.add_argument("--cpu-blocks", type=int, default=4)
    ap.add_argument("--profile-case", action="store_true",
                    help="n=20000, p=20000 case of the same subset shape, for ncu captures")
    ap.add_argument("--precision", default="fp8", choices=["fp64", "fp32", "fp8"], help="--profile-case only")
    ap.add_argument("--workload", default="c3", choices=["c3", "c5"],
                    help="c5: config 5 (BayesRc, n=50000, p=1000000, 16 chains) on its own JSON line")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
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
                "scaling": "weak", "vs_baseline": None, "dtype": "u8 genotypes x f32 (FP8-exact codes, FP32 "
                                                                  "accumulation, FP64 draws)",
                "data": "synthetic (seeded generator of config 3)",
                "config": {**config, "chains": args.chains, "precision": "fp8", "settle_iterations": args.settle,
                           "parallelism": f"replicas x{ws}"},
                "fp32_plain": res["fp32_plain"],
                "speedup_vs_fp32_plain": res["value"] / ws / res["fp32_plain"]["value"],
                "error_vs_fp64": res["error_vs_fp64"], "roofline": res["roofline"], "roofline_rhs": res["roofline_rhs"],
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
                "included_at_timing": res["included_at_timing"]}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
