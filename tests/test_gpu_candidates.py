"""Candidate correction (correct_candidates) and the combine step on the GPU.

HQ anchors correct the candidates of their final MSA; cg_combine_results then
keeps a low-quality anchor correction only where all of its two or more
candidate corrections agree with it (reference: src/msa.cpp:457-522,
include/corrector.hpp:1504-1512 and 1674-1748,
src/correctionresultoutput.cpp:1256-1551).  The reference's own outputs for
this mode are fixtures (se_candidates, pe_candidates,
se_candidates_varlen_quality, se_candidates_tail; checked by the fixture tests
of test_gpu_parity.py, test_gpu_batched.py and test_gpu_files.py); here the
oracle, pinned to those fixtures, checks the paths they do not reach: reads
longer than 256 bp (the block-per-anchor MSA), the forest decision, a wide
new_columns_to_correct, passes over several calls, the batched driver and the
learned decision.
"""
import numpy as np
import pytest

import fixtures as fx
import oracle
from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu

C = capi


def gpu_run(opts, r, quality=False, forest=None, trees=0):
    g = capi.CareGpu(opts)
    g.append_reads(r.sequences, r.offsets, r.qualities if quality else None)
    g.build_tables()
    if forest:
        g.load_forest(forest, trees)
    flags, seqs = g.correct()
    st = g.stats()
    g.close()
    return flags, seqs, st


def oracle_run(opts, r, quality=False, forest=None, trees=0):
    orc = oracle.Oracle(opts, r.sequences, r.offsets, r.qualities if quality else None)
    if forest:
        orc.load_forest(forest, trees if trees else 0xFFFFFFFF, opts.threshold_anchor)
    return orc.correct()


def assert_same(r, flags, seqs, oflags, oseqs):
    assert np.array_equal(flags, oflags), f"{int((flags != oflags).sum())} reads differ in flags"
    lens = r.lengths
    idx = np.nonzero(flags & C.CG_RESULT_CORRECTED)[0]
    bad = [int(i) for i in idx if not np.array_equal(seqs[i, :lens[i]], oseqs[i, :lens[i]])]
    assert not bad, f"{len(bad)} corrected reads differ, first {bad[:5]}"


def repeats(seed, n=8_000, **kw):
    cfg = sim.SimConfig(seed=seed, genome_length=40_000, repeat_families=4, repeat_copies=4, repeat_min_len=800,
                        repeat_max_len=2500, num_reads=n, sub_rate_5p=0.002, sub_rate_3p=0.02, **kw)
    return sim.SimReads(cfg)


def cand_opts(**kw):
    return capi.CareOptions.defaults(30.0, correct_candidates=1, **kw)


def test_combine_outcomes_all_occur_and_match_oracle():
    r = repeats(61)
    flags, seqs, st = gpu_run(cand_opts(), r)
    oflags, oseqs, ocnt = oracle_run(cand_opts(), r)
    assert_same(r, flags, seqs, oflags, oseqs)
    for bit in (C.CG_RESULT_CANDIDATES, C.CG_RESULT_REJECTED, C.CG_RESULT_CANDIDATE_RECORD):
        assert (flags & bit).any(), bit
    assert st["candidate_corrections"] > 0


@pytest.mark.parametrize("quality", [False, True])
def test_long_reads_match_oracle(quality):
    # reads up to 400 bp: alignment and MSA take the block-per-anchor kernels
    r = repeats(62, n=5_000, read_len_min=180, read_len_max=400)
    opts = cand_opts(use_quality_scores=int(quality))
    flags, seqs, _ = gpu_run(opts, r, quality)
    oflags, oseqs, _ = oracle_run(cand_opts(use_quality_scores=int(quality)), r, quality)
    assert_same(r, flags, seqs, oflags, oseqs)
    assert (flags & C.CG_RESULT_CANDIDATES).any()


def test_long_reads_without_candidates_match_oracle():
    r = repeats(63, n=5_000, read_len_min=120, read_len_max=330)
    kw = dict(use_quality_scores=1)
    flags, seqs, _ = gpu_run(capi.CareOptions.defaults(30.0, **kw), r, True)
    oflags, oseqs, _ = oracle_run(capi.CareOptions.defaults(30.0, **kw), r, True)
    assert_same(r, flags, seqs, oflags, oseqs)


def test_forest_decision_with_candidates_matches_oracle():
    forest = fx.forest_bytes(fx.manifest()["forest_se"])
    r = repeats(64)
    kw = dict(correction_type=C.CG_CORR_FOREST, threshold_anchor=0.6)
    flags, seqs, _ = gpu_run(cand_opts(**kw), r, forest=forest, trees=5)
    oflags, oseqs, _ = oracle_run(cand_opts(**kw), r, forest=forest, trees=5)
    assert_same(r, flags, seqs, oflags, oseqs)


@pytest.mark.parametrize("nc", [0, 40])
def test_new_columns_to_correct(nc):
    # 0: only candidates within the anchor's columns; 40: the extension
    # columns of the warp MSA span two lane groups
    r = repeats(65, read_len_min=100, read_len_max=150)
    flags, seqs, _ = gpu_run(cand_opts(new_columns_to_correct=nc), r)
    oflags, oseqs, _ = oracle_run(cand_opts(new_columns_to_correct=nc), r)
    assert_same(r, flags, seqs, oflags, oseqs)


def test_batched_driver_matches_plain():
    r = repeats(66, n=12_000)
    plain = gpu_run(cand_opts(), r)
    o = cand_opts(driver=C.CG_DRIVER_BATCHED, batch_anchors=2048, msa_warps=2, streams=2)
    bat = gpu_run(o, r)
    assert_same(r, bat[0], bat[1], plain[0], plain[1])
    assert bat[2]["candidate_corrections"] == plain[2]["candidate_corrections"]


def test_batched_driver_with_autotuning_matches_plain():
    # enough anchors for the tuner (a read count of its own, so that no earlier
    # test's tuned shape is reused): its trials must not vote
    cfg = sim.SimConfig(seed=70, genome_length=700_000, repeat_families=20, repeat_copies=4, num_reads=140_000,
                        sub_rate_5p=0.002, sub_rate_3p=0.02)
    r = sim.SimReads(cfg)
    plain = gpu_run(cand_opts(), r)
    bat = gpu_run(cand_opts(driver=C.CG_DRIVER_BATCHED), r)
    assert_same(r, bat[0], bat[1], plain[0], plain[1])
    assert bat[2]["candidate_corrections"] == plain[2]["candidate_corrections"]


def test_pass_over_several_calls_and_repeated_passes():
    r = repeats(67)
    n = r.n
    g = capi.CareGpu(cand_opts(batch_anchors=1500))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    whole, wseqs = g.correct()
    # the same pass split into three calls, then combined
    parts = [(0, 3000), (3000, 2500), (5500, n - 5500)]
    flags = np.zeros(n, np.uint8)
    seqs = np.zeros_like(wseqs)
    for f, c in parts:
        pf, ps = g.correct(f, c)
        flags[f:f + c], seqs[f:f + c] = pf, ps
    assert not (flags & (C.CG_RESULT_CANDIDATES | C.CG_RESULT_REJECTED)).any()  # not combined yet
    recs = g.combine(0, flags)
    assert recs > 0
    assert_same(r, flags, seqs, whole, wseqs)
    # a repeated full call starts a new pass: same result, votes not doubled
    again, aseqs = g.correct()
    assert_same(r, again, aseqs, whole, wseqs)
    # combining a sub-range gives the same flags as that part of the whole
    sub = np.zeros(2000, np.uint8)
    pf, _ = g.correct(0, n, combine=False)
    sub[:] = pf[1000:3000]
    g.combine(1000, sub)
    assert np.array_equal(sub, whole[1000:3000])
    g.close()


def test_learned_decision_with_candidates_batched_matches_plain():
    # the learned decision has no reference counterpart: both drivers must
    # agree, and only LQ corrections may be kept or rejected by the combine
    from rabbitqcplus_gb300 import learned
    model = open(learned.DEFAULT_MODEL, "rb").read()
    r = repeats(69, n=10_000)
    res = []
    for drv in (C.CG_DRIVER_PLAIN, C.CG_DRIVER_BATCHED):
        o = cand_opts(correction_type=C.CG_CORR_LEARNED, driver=drv, batch_anchors=2048)
        g = capi.CareGpu(o)
        g.append_reads(r.sequences, r.offsets)
        g.build_tables()
        g.load_classifier(model)
        res.append(g.correct())
        g.close()
    (pf, ps), (bf, bs) = res
    assert_same(r, bf, bs, pf, ps)
    lq = (pf & C.CG_RESULT_CORRECTED) != 0
    lq &= (pf & C.CG_RESULT_HQ) == 0
    combined = (pf & (C.CG_RESULT_CANDIDATES | C.CG_RESULT_REJECTED)) != 0
    assert combined.any() and not (combined & ~lq).any()


def test_combine_needs_candidate_correction():
    r = repeats(68, n=2_000)
    g = capi.CareGpu(capi.CareOptions.defaults(30.0))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    flags, _ = g.correct()
    with pytest.raises(capi.CareError):
        g.combine(0, flags)
    g.close()
