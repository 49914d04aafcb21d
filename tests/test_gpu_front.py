"""Front-end on the GPU: the device tokeniser (subby_tokenize) against the
host lookup, its first-bad-character report, JSON requests
(subby_gb300.io.run) against the reference's own io.run outputs (FP64
oracle) stored in tests/golden/formats/formats.json, and the MAF batch
pipeline (subby_gb300.maf_batch) against the reference batch script's
outputs in tests/golden/maf.  Tolerances as everywhere (tests/_tol.py)."""
import json
import os

import numpy as np
import pytest

from tests._tol import COUNTS_RTOL, ROOTPROB_RTOL, assert_cols, assert_loglike

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from subby_gb300 import formats, io, maf_batch  # noqa: E402

with open(os.path.join(os.path.dirname(__file__), "golden", "formats", "formats.json")) as f:
    G = json.load(f)


@pytest.mark.parametrize("shape", [(3, 17), (7, 1000), (64, 4099), (1, 1), (3, 0)])
def test_device_tokenizer_matches_host(shape):
    rng = np.random.default_rng(shape[1])
    alphabet = list("ACGT")
    chars = rng.choice(np.frombuffer(b"ACGTacgt-.", dtype=np.uint8), size=shape)
    host = formats.tokenize(chars, alphabet)
    dev = formats.tokenize(torch.as_tensor(chars).cuda(), alphabet)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    assert host.size == 0 or (0 <= host.min() and host.max() <= 5)


def test_device_tokenizer_reports_first_bad_character():
    chars = np.frombuffer(b"ACGT" * 100, dtype=np.uint8).copy().reshape(4, 100)
    chars[2, 37] = ord("X")
    chars[3, 90] = ord("Z")
    with pytest.raises(ValueError, match=r"Unknown character 'X' at row 2, col 37"):
        formats.tokenize(torch.as_tensor(chars).cuda(), list("ACGT"))


def test_large_device_tokenization():
    n_rows, C = 255, 1 << 20
    rng = np.random.default_rng(1)
    chars = torch.as_tensor(rng.choice(np.frombuffer(b"ACGT-", dtype=np.uint8), size=(n_rows, C))).cuda()
    tok = formats.tokenize(chars, list("ACGT"))
    torch.cuda.synchronize()
    sample = chars[:, ::4099].cpu().numpy()
    np.testing.assert_array_equal(tok[:, ::4099].cpu().numpy(), formats.tokenize(sample, list("ACGT")))


@pytest.mark.parametrize("case", G["requests"], ids=lambda c: c["request"]["model"].get("name", "subRate"))
def test_requests_match_reference_io(case):
    got = io.run(case["request"])
    ref = case["result"]
    assert set(got) == set(ref)
    if "logLike" in ref:
        assert_loglike(np.array(got["logLike"]), np.array(ref["logLike"]))
    if "counts" in ref:
        assert_cols(np.array(got["counts"]), np.array(ref["counts"]), COUNTS_RTOL, "counts")
        assert_cols(np.array(got["dwellTimes"]), np.array(ref["dwellTimes"]), COUNTS_RTOL, "dwell")
    if "rootProb" in ref:
        assert_cols(np.array(got["rootProb"]), np.array(ref["rootProb"]), ROOTPROB_RTOL, "rootProb")


def test_command_line_runs_a_request(tmp_path):
    """``python -m subby_gb300 request.json -o out.json`` (subby/__main__.py)
    writes the reference io.run result, within the usual tolerances."""
    import subprocess
    import sys
    case = G["requests"][0]
    req = tmp_path / "req.json"
    req.write_text(json.dumps(case["request"]))
    out = tmp_path / "out.json"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run([sys.executable, "-m", "subby_gb300", str(req), "-o", str(out), "--indent", "1"], check=True,
                   cwd=root)
    got, ref = json.loads(out.read_text()), case["result"]
    assert set(got) == set(ref)
    assert_loglike(np.array(got["logLike"]), np.array(ref["logLike"]))
    assert_cols(np.array(got["counts"]), np.array(ref["counts"]), COUNTS_RTOL, "counts")
    assert_cols(np.array(got["rootProb"]), np.array(ref["rootProb"]), ROOTPROB_RTOL, "rootProb")


def test_maf_batch_pipeline(tmp_path):
    """The command line of the MAF batch pipeline on the GPU: manifest,
    per-block files and diagnostics as the reference script wrote them;
    features within the Counts tolerance, column by column."""
    d = os.path.join(os.path.dirname(__file__), "golden", "maf")
    with open(os.path.join(d, "expected.json")) as f:
        E = json.load(f)
    Z = np.load(os.path.join(d, "expected.npz"))
    out = tmp_path / "out"
    maf_batch.main([os.path.join(d, "blocks.maf"), str(out), "--tree", os.path.join(d, "guide.nh"),
                    "--exclude-species", ",".join(E["exclude"]), "--min-species", str(E["min_species"]),
                    "--min-cols", str(E["min_cols"]), "--max-cols", str(E["max_cols"]),
                    "--kappa", str(E["kappa"]), "--pi", ",".join(map(str, E["pi"])),
                    "--validate", str(E["validate"])])
    with open(out / "manifest.json") as f:
        man = json.load(f)
    assert man == E["manifest"]
    for m, meta in zip(man, E["per_block"]):
        z = np.load(out / m["file"])
        assert z["species"].tolist() == meta["species"]
        assert (int(z["n_species"]), int(z["n_species_original"]), int(z["length"])) == \
            (meta["n_species"], meta["n_species_original"], meta["length"])
        assert z["features"].dtype == np.float32
        assert_cols(z["features"].T, Z[m["file"][:-4]].T, COUNTS_RTOL, m["file"])
    with open(out / "validation_diagnostics.json") as f:
        diag = json.load(f)
    assert len(diag) == len(E["diagnostics"])
    for got, exp in zip(diag, E["diagnostics"]):
        for k in ("block_idx", "n_species", "n_cols", "n_species_excluded"):
            assert got[k] == exp[k]
        for k in ("mean_trans_matrix", "symmetry_ratio", "total_dwell_per_col", "ti_tv_ratio", "count_cv",
                  "total_counts_mean", "total_counts_std"):
            np.testing.assert_allclose(got[k], exp[k], rtol=1e-3, atol=1e-6, err_msg=k)
