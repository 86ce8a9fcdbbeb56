"""Generates the golden fixtures in this directory from the reference's shipped
example files (run once where the reference checkout is available; the
fixtures are committed, the tests never read the reference).

Usage: python tests/golden/make_golden.py <reference checkout>

pred_kat.npz — prediction known-answer test.  The reference's prediction
    mode (SODABayes.f90:145-148 -> setup_prediction, xscale, compute_dgv,
    write_dgv) applied to examples/data/simdata1_pred.bed with the shipped
    .frq/.eff/.mod of examples 1, 3 and 4 produced the shipped pred_*.gv files.
    The fixture keeps the first NKEEP individuals: their 2-bit genotype
    records (re-packed), the three effect sets, the allele frequencies, the
    three means and the three expected .gv columns (E15.7 text values).
formats.json — verbatim lines of the shipped .hyp/.eff/.mod/.frq/.gv/.log
    files of example 1 and the .eff/.mod header lines of examples 2 and 4,
    used to pin the output writers byte for byte.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EX = ""   # <reference checkout>/examples, set from the command line
NKEEP = 100
NIND, NLOCI = 900, 9346


def read_bed_codes(path, nind, nloci):
    raw = np.fromfile(path, dtype=np.uint8)
    assert raw[0] == 0x6C and raw[1] == 0x1B and raw[2] == 1
    rec = (nind + 3) // 4
    b = raw[3:].reshape(nloci, rec)
    codes2 = np.stack([(b >> (2 * k)) & 3 for k in range(4)], axis=2).reshape(nloci, -1)[:, :nind]
    return codes2.astype(np.uint8)   # raw 2-bit PLINK codes, SNP-major


def repack(codes2):
    nloci, nind = codes2.shape
    rec = (nind + 3) // 4
    pad = np.zeros((nloci, rec * 4), dtype=np.uint8)
    pad[:, :nind] = codes2
    q = pad.reshape(nloci, rec, 4)
    return (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)


def main():
    codes2 = read_bed_codes(os.path.join(EX, "data", "simdata1_pred.bed"), NIND, NLOCI)
    kept = codes2[:, :NKEEP]
    sets = [("example1/bayesr_mcmc_example_1", "example1/pred_bayesr_mcmc_example_1"),
            ("example3/bayesr_mcmc_example_2", "example3/pred_bayesr__example_3"),
            ("example4/bayesrc_mcmc_example_4", "example4/pred_bayesrc_mcmc_example_4")]
    effs, mus, gvs, ids, frqs = [], [], [], [], []
    for model, pred in sets:
        eff = np.loadtxt(os.path.join(EX, model + ".eff"), skiprows=1, usecols=1)
        frq = np.loadtxt(os.path.join(EX, model + ".frq"), usecols=1)
        mu = float(open(os.path.join(EX, model + ".mod")).read().split()[1])
        gv = np.loadtxt(os.path.join(EX, pred + ".gv"), usecols=1)[:NKEEP]
        gid = np.loadtxt(os.path.join(EX, pred + ".gv"), usecols=0, dtype=np.int64)[:NKEEP]
        effs.append(eff)
        frqs.append(frq)
        mus.append(mu)
        gvs.append(gv)
        ids.append(gid)
    for f in frqs[1:]:
        assert np.array_equal(f, frqs[0]), "the three models share the training frequencies"
    np.savez_compressed(os.path.join(HERE, "pred_kat.npz"), bed=repack(kept), nind=NKEEP, nloci=NLOCI,
                        freq=frqs[0], eff=np.stack(effs), mu=np.array(mus), gv=np.stack(gvs), ids=ids[0])
    fm = {}
    e1 = os.path.join(EX, "example1", "bayesr_mcmc_example_1")
    with open(e1 + ".hyp") as f:
        fm["hyp_bayesr"] = [next(f) for _ in range(4)]
    with open(e1 + ".eff") as f:
        fm["eff_bayesr"] = [next(f) for _ in range(4)]
    with open(e1 + ".frq") as f:
        fm["frq"] = [next(f) for _ in range(4)]
    with open(e1 + ".mod") as f:
        fm["mod_bayesr"] = f.readlines()
    with open(e1 + ".gv") as f:
        fm["gv"] = [next(f) for _ in range(4)]
    with open(e1 + ".log") as f:
        fm["log_bayesr"] = f.readlines()
    e4 = os.path.join(EX, "example4", "bayesrc_mcmc_example_4")
    with open(e4 + ".mod") as f:
        fm["mod_bayesrc"] = f.readlines()
    with open(e4 + ".hyp") as f:
        fm["hyp_bayesrc"] = [next(f) for _ in range(3)]
    with open(os.path.join(EX, "example1", "pred_bayesr_mcmc_example_1.log")) as f:
        fm["log_predict"] = f.readlines()
    with open(os.path.join(EX, "example2", "bayesr_mcmc_example_2.log")) as f:
        fm["log_sodaoff"] = f.readlines()
    with open(os.path.join(HERE, "formats.json"), "w") as f:
        json.dump(fm, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout (the directory holding examples/)>")
    EX = os.path.join(sys.argv[1], "examples")
    main()
