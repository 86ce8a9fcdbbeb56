"""Golden vectors from the reference's shipped examples (see tests/golden/make_golden.py).

The prediction known-answer test pins the bed decode (utilities.f90:438-454),
the prediction branch of xscale (540-553) and compute_dgv (616-622): the
reference wrote the expected values with format E15.7, so agreement is to
half a unit in the 8th significant digit."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def kat():
    return np.load(os.path.join(GOLD, "pred_kat.npz"))


def _tol(gv):
    return 0.5e-7 * 10.0 ** np.ceil(np.log10(np.abs(gv))) + 1e-12


def test_oracle_prediction_matches_reference_outputs(oracle_mod, kat):
    n, p = int(kat["nind"]), int(kat["nloci"])
    codes = oracle_mod.decode_bed(kat["bed"], n, p)
    assert set(np.unique(codes)) <= {0, 1, 2}
    for s in range(3):
        pred = oracle_mod.predict(codes, kat["freq"], kat["mu"][s], kat["eff"][s])
        assert np.all(np.abs(pred - kat["gv"][s]) <= _tol(kat["gv"][s])), s


def test_bed_decode_maps_missing_to_het(oracle_mod):
    # one SNP, four individuals with codes 00, 01 (missing), 10, 11
    payload = np.array([0b11100100], dtype=np.uint8)
    codes = oracle_mod.decode_bed(payload, 4, 1)
    assert codes[:, 0].tolist() == [0, 1, 1, 2]


@pytest.mark.gpu
def test_gpu_prediction_matches_reference_outputs(gpu_lib, kat):
    import sodabayes_gb300 as sg
    n, p = int(kat["nind"]), int(kat["nloci"])
    for s in range(3):
        pred = sg.predict(bed=kat["bed"], nind=n, freq=kat["freq"], mu=kat["mu"][s], effects=kat["eff"][s])
        assert np.all(np.abs(pred - kat["gv"][s]) <= _tol(kat["gv"][s])), s


@pytest.mark.gpu
def test_gpu_prediction_matches_oracle(gpu_lib, oracle_mod, kat):
    import sodabayes_gb300 as sg
    n, p = int(kat["nind"]), int(kat["nloci"])
    codes = oracle_mod.decode_bed(kat["bed"], n, p)
    for s in range(3):
        want = oracle_mod.predict(codes, kat["freq"], kat["mu"][s], kat["eff"][s])
        got = sg.predict(codes=codes, freq=kat["freq"], mu=kat["mu"][s], effects=kat["eff"][s])
        assert np.allclose(got, want, rtol=1e-12, atol=1e-10)


@pytest.mark.gpu
def test_gpu_prediction_rejects_codes_outside_0_to_2(gpu_lib, kat):
    """Codes other than 0/1/2 are an argument error in prediction mode, as
    when loading genotypes (the centring table has three values per SNP)."""
    import sodabayes_gb300 as sg
    n, p = 50, 40
    codes = np.ones((n, p), dtype=np.int8)
    freq = np.full(p, 0.5)
    eff = np.ones(p)
    assert np.allclose(sg.predict(codes=codes, freq=freq, mu=1.0, effects=eff), 1.0)
    for bad in (-1, 3, -9):
        c2 = codes.copy()
        c2[7, 3] = bad
        with pytest.raises(sg.SodaGpuError) as ei:
            sg.predict(codes=c2, freq=freq, mu=1.0, effects=eff)
        assert ei.value.code == -1
