"""The `sodabayes` job driver (sodabayes_gb300/csrc/host): Fortran edit
descriptors checked against the reference's own output files
(tests/golden/formats.json), option and .par handling, and on the GPU a
two-job .par run (BayesR MCMC, then prediction) whose files must have the
reference's layout byte for byte (headers, labels, field widths) and
numbers consistent with the model (.gv = mu + X g)."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "sodabayes_gb300", "sodabayes")
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "formats.json")))


@pytest.fixture(scope="module")
def cli():
    from sodabayes_gb300 import build
    build.build()
    assert os.path.exists(CLI)
    return CLI


def _fmt(cli, v):
    out = subprocess.run([cli, "--format-selftest", repr(v)], capture_output=True, text=True, check=True).stdout
    return dict(re.findall(r"(\w+\.\d+|I12)\[([^\]]*)\]", out))


def test_e_format_reproduces_reference_outputs(cli):
    toks = set()
    for key in ("hyp_bayesr", "eff_bayesr", "mod_bayesr", "mod_bayesrc", "hyp_bayesrc"):
        for line in GOLDEN[key][1:] if key.startswith(("hyp", "eff")) else GOLDEN[key]:
            toks.update(re.findall(r"-?0\.\d{6}E[+-]\d\d", line))
    gv = {t for line in GOLDEN["gv"] for t in re.findall(r"-?0\.\d{7}E[+-]\d\d", line)}
    assert len(toks) > 50 and len(gv) >= 3
    for t in sorted(toks)[:400]:
        assert _fmt(cli, float(t))["E15.6"] == t.rjust(15), t
    for t in gv:
        assert _fmt(cli, float(t))["E15.7"] == t.rjust(15), t


def test_f_format_reproduces_frq(cli):
    for line in GOLDEN["frq"]:
        t = line.split()[1]
        assert _fmt(cli, float(t))["F10.6"] == t.rjust(10)
        assert line == line[:10] + " " + t.rjust(10) + "\n"


def test_help_and_option_errors(cli, tmp_path):
    out = subprocess.run([cli, "-h"], capture_output=True, text=True).stdout
    assert out.splitlines()[0].startswith("argument    type        description")
    assert any(l.startswith("-method     [char]      Bayesian method") for l in out.splitlines())
    par = tmp_path / "job.par"
    par.write_text("# comment\nBEGIN my job\n  -bfile nowhere   # trailing comment\n  -method BayesR\nEND my job\n")
    r = subprocess.run([cli, str(par)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1
    assert "job my job started..." in r.stdout
    assert "plink file nowhere.bed not found" in r.stdout
    assert "job my job did not complete." in r.stdout
    r = subprocess.run([cli, "-bfile", "x", "-bogus", "1"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "Unknown command line option : -bogus" in r.stdout
    r = subprocess.run([cli, "-bfile", "-method"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "Missing argument for :-bfile" in r.stdout


def write_plink(prefix, codes, y):
    """SNP-major .bed (code 0 -> 00, 1 -> 10, 2 -> 11), .bim, .fam."""
    n, p = codes.shape
    bits = {0: 0b00, 1: 0b10, 2: 0b11}
    rec = (n + 3) // 4
    out = bytearray(b"\x6c\x1b\x01")
    for j in range(p):
        row = bytearray(rec)
        for i in range(n):
            row[i // 4] |= bits[int(codes[i, j])] << (2 * (i % 4))
        out += row
    open(prefix + ".bed", "wb").write(bytes(out))
    with open(prefix + ".bim", "w") as f:
        for j in range(p):
            f.write(f"1 snp{j + 1} 0 {j + 1} A G\n")
    with open(prefix + ".fam", "w") as f:
        for i in range(n):
            f.write(f"fam{i + 1} ind{i + 1} 0 0 1 {y[i]:.6f}\n")


@pytest.mark.gpu
def test_cli_two_jobs_match_reference_layout(cli, gpu_lib, tmp_path):
    from sodabayes_gb300 import synth
    n, p = 300, 900
    G, y, _ = synth.make(synth.SynthSpec(n=n, p=p, ld_block=25, rho=0.5, ncausal=30, h2=0.5, mean=50.0, seed=3))
    write_plink(str(tmp_path / "train"), G, y)
    write_plink(str(tmp_path / "pred"), G[:120], y[:120])
    (tmp_path / "ex.par").write_text(
        "#two jobs\n"
        "BEGIN CLI_BayesR_MCMC\n"
        "   -bfile train\n   -method BayesR\n   -scale_va 50\n   -scale_ve 50\n   -df_va 4.5\n   -df_ve 4.5\n"
        "   -numit 40\n   -burnin 10\n   -thin 1\n   -nmix 4\n   -mix 0.0,0.0001,0.001,0.01\n   -SODAOn\n"
        "   -nthreads 4\n   -nblocks 3\n   -seed 123456789\n   -out bayesr_cli\n"
        "END CLI_BayesR_MCMC\n\n"
        "BEGIN CLI_Prediction\n   -bfile pred\n   -predict\n   -model bayesr_cli.mod\n   -freq bayesr_cli.frq\n"
        "   -effects bayesr_cli.eff\n   -out pred_cli\nEND CLI_Prediction\n")
    r = subprocess.run([cli, "ex.par"], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "job CLI_BayesR_MCMC completed." in r.stdout and "job CLI_Prediction completed." in r.stdout
    # .hyp: header identical to the reference's, 40 rows in its field widths (trailing blank included)
    hyp = open(tmp_path / "bayesr_cli.hyp").readlines()
    assert hyp[0] == GOLDEN["hyp_bayesr"][0]
    assert len(hyp) == 41
    ref_row = GOLDEN["hyp_bayesr"][1]
    for row in hyp[1:]:
        assert len(row) == len(ref_row) and row.endswith(" \n")
        assert re.fullmatch(r"( {0,11}\d{1,12}){2}( {1,4}-?0\.\d{6}E[+-]\d\d){3}( {1,12}\d{1,12}){4}"
                            r"( {1,5}-?0\.\d{6}E[+-]\d\d){4} \n", row), row
    assert [int(l.split()[0]) for l in hyp[1:]] == list(range(1, 41))
    # .eff: header identical; one row per SNP in (A10,1X,E15.6,4(1X,E15.6))
    eff = open(tmp_path / "bayesr_cli.eff").readlines()
    assert eff[0] == GOLDEN["eff_bayesr"][0]
    assert len(eff) == p + 1 and all(len(l) == 10 + 5 * 16 + 1 for l in eff[1:])
    assert eff[1].startswith("snp1      ")
    # .mod: the reference's labels in its order and layout (a,t10,E15.6)
    mod = open(tmp_path / "bayesr_cli.mod").readlines()
    assert [l[:9] for l in mod] == [l[:9] for l in GOLDEN["mod_bayesr"]]
    assert all(len(l) == 25 for l in mod)
    # .frq: (A10,1X,F10.6), equal to the genotype frequencies
    frq = open(tmp_path / "bayesr_cli.frq").readlines()
    f_np = G.sum(axis=0) / (2.0 * n)
    assert len(frq) == p and all(len(l) == 22 for l in frq)
    assert np.allclose([float(l.split()[1]) for l in frq], f_np, atol=5e-7)
    # .gv: (A20,1x,E15.7) and equal to mean + X * effects of the written model
    gv = open(tmp_path / "bayesr_cli.gv").readlines()
    assert len(gv) == n and all(len(l) == 37 and l.startswith("ind") for l in gv)
    mu = float(mod[0].split()[1])
    g = np.array([float(l.split()[1]) for l in eff[1:]])
    ok = (f_np > np.finfo(float).eps) & (1 - f_np > np.finfo(float).eps)
    X = np.where(ok, (G - 2 * f_np) / np.sqrt(2 * f_np * (1 - f_np) + (~ok)), 0.0)
    pred = mu + X @ g
    got = np.array([float(l.split()[1]) for l in gv])
    assert np.max(np.abs(got - pred)) <= 1e-5 * np.max(np.abs(pred))
    # prediction job: the first 120 individuals again, from the written (rounded) .frq/.eff/.mod
    pgv = open(tmp_path / "pred_cli.gv").readlines()
    assert len(pgv) == 120
    assert np.allclose([float(l.split()[1]) for l in pgv], got[:120], rtol=2e-5)
    # .log: the reference's labels and layout
    log = open(tmp_path / "bayesr_cli.log").readlines()
    ref_log = GOLDEN["log_bayesr"]
    assert log[0] == "Running program SODABayes: CLI_BayesR_MCMC\n"
    assert log[1].startswith("      Run started at ")
    labels = [l[:31] for l in ref_log[2:21]]
    assert [l[:31] for l in log[2:21]] == labels
    assert log[16] == "No. of blocks                =        3\n"
    assert log[20] == "Prefix for output files      : bayesr_cli\n"
    assert log[-3].startswith("        Run ended at ") and log[-2] == "        Walltime used (seconds)\n"
    assert log[-1].startswith("Setup: ") and " MCMC: " in log[-1] and " Total: " in log[-1]
    plog = open(tmp_path / "pred_cli.log").readlines()
    assert [l[:31] for l in plog[2:9]] == [l[:31] for l in GOLDEN["log_predict"][2:9]]


@pytest.mark.gpu
def test_cli_sodaoff_runs_the_regular_sampler(cli, gpu_lib, tmp_path):
    """-SODAOff (SODABayes.f90:134-137): regular_bayes on the GPU; the .log has
    the reference's example-2 layout ('SODA off = T', no block lines) and the
    .hyp its rows."""
    from sodabayes_gb300 import synth
    n, p = 200, 300
    G, y, _ = synth.make(synth.SynthSpec(n=n, p=p, ld_block=25, rho=0.5, ncausal=20, h2=0.5, mean=50.0, seed=4))
    write_plink(str(tmp_path / "train"), G, y)
    (tmp_path / "off.par").write_text(
        "BEGIN BayesR_Regular_MCMC\n"
        "   -bfile train\n   -method BayesR\n   -scale_va 50\n   -scale_ve 50\n   -df_va 4.5\n   -df_ve 4.5\n"
        "   -numit 30\n   -burnin 10\n   -thin 1\n   -nmix 4\n   -mix 0.0,0.0001,0.001,0.01\n   -SODAOff\n"
        "   -seed 123456789\n   -out bayesr_off\n"
        "END BayesR_Regular_MCMC\n")
    r = subprocess.run([cli, "off.par"], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    log = open(tmp_path / "bayesr_off.log").readlines()
    ref = GOLDEN["log_sodaoff"]
    assert log[0] == "Running program SODABayes: BayesR_Regular_MCMC\n"
    assert [l[:31] for l in log[2:17]] == [l[:31] for l in ref[2:17]]
    assert log[14] == "SODA off                     = T\n"
    hyp = open(tmp_path / "bayesr_off.hyp").readlines()
    assert hyp[0] == GOLDEN["hyp_bayesr"][0] and len(hyp) == 31
    eff = open(tmp_path / "bayesr_off.eff").readlines()
    assert len(eff) == p + 1
