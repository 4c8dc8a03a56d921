"""Pins the oracle (CPU restatement) to fixtures produced by the reference.

The fixtures in tests/golden/ were made by tests/golden/make_golden.py, which
ran the reference's own care::performCorrection (compiled from its sources by
oracle/ref.mk) and its per-stage internals (oracle/ref_stages.cpp).  These
tests need no GPU.
"""
import struct

import numpy as np
import pytest

import fixtures as fx
import oracle
from rabbitqcplus_gb300 import capi


def f2b(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


@pytest.fixture(scope="module")
def cases():
    return fx.manifest()


@pytest.mark.parametrize("name", fx.case_names())
def test_generator_is_deterministic(name, cases):
    e = cases[name]
    r = fx.reads_for(e)
    assert r.n == e["num_reads"]
    assert fx.md5(r.sequences) == e["input_md5"]
    assert fx.md5(r.qualities) == e["input_qual_md5"]


@pytest.mark.parametrize("name", fx.case_names())
def test_oracle_output_matches_reference(name, cases):
    e = cases[name]
    r = fx.reads_for(e)
    opts = fx.options_for(e)
    q = r.qualities if e["options"].get("quality") else None
    orc = oracle.Oracle(opts, r.sequences, r.offsets, q, threads=4)
    if fx.forest_bytes(e):
        orc.load_forest(fx.forest_bytes(e))
    flags, seqs, _ = orc.correct()
    out = capi.apply_corrections(r.sequences, r.offsets, flags, seqs)
    exp = fx.expected_output(name, r)
    assert fx.md5(exp) == e["output_md5"]
    bad = np.nonzero(out != exp)[0]
    assert bad.size == 0, f"{bad.size} bases differ from the reference"
    assert r.score(out) == e["score"]


STAGE_CASES = [n for n in fx.case_names() if fx.manifest()[n].get("stage_anchors")]


@pytest.mark.parametrize("name", STAGE_CASES)
def test_oracle_signatures_and_candidates_match_reference(name, cases):
    e = cases[name]
    r = fx.reads_for(e)
    orc = oracle.Oracle(fx.options_for(e), r.sequences, r.offsets,
                        r.qualities if e["options"].get("quality") else None, threads=4)
    st = fx.load_stages(name)
    ids = sorted(st["sigs"])
    sig = orc.signatures(0, len(ids))
    for i in ids:
        assert sig[i].tolist() == st["sigs"][i], f"signature of read {i}"
    for a in st["anchors"]:
        assert orc.candidates(a["id"]).tolist() == a["cand"], f"candidates of anchor {a['id']}"


@pytest.mark.parametrize("name", STAGE_CASES)
def test_oracle_anchor_corrections_match_reference_stages(name, cases):
    e = cases[name]
    r = fx.reads_for(e)
    orc = oracle.Oracle(fx.options_for(e), r.sequences, r.offsets,
                        r.qualities if e["options"].get("quality") else None, threads=4)
    st = fx.load_stages(name)
    n = len(st["anchors"])
    flags, seqs, _ = orc.correct(0, n)
    for a in st["anchors"]:
        i = a["id"]
        if "corr" not in a:
            assert flags[i] == 0, f"anchor {i} should have no correction"
            continue
        corrected, text = a["corr"]
        assert bool(flags[i] & capi.CG_RESULT_CORRECTED) == bool(corrected)
        assert bool(flags[i] & capi.CG_RESULT_HQ) == bool(a["prop"][4]) or not corrected
        if corrected:
            assert seqs[i, :a["len"]].tobytes().decode() == text
