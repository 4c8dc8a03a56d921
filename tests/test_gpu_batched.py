"""The batched driver (captured batch graphs, persistent work-stealing
kernels, autotuned shapes) gives results identical to the plain driver.

Both drivers run the same per-candidate and per-anchor computations; only the
order in which blocks take their work differs.  So the bar is bit-exact:
identical flags, identical corrected bases and identical pipeline counters.
"""
import numpy as np
import pytest

import fixtures as fx
from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu

COUNTERS = ("raw_candidate_ids", "unique_candidates", "aligned_candidates", "msa_candidates", "msa_builds",
            "corrected_anchors", "hq_anchors")


def run(opts, reads, quality=False, forest=None, first=0, count=None, repeat=1):
    g = capi.CareGpu(opts)
    g.append_reads(reads.sequences, reads.offsets, reads.qualities if quality else None)
    g.build_tables()
    if forest:
        g.load_forest(forest)
    res = [g.correct(first, count) for _ in range(repeat)]
    st = g.stats()
    g.close()
    return res, st


def batched(opts, batch, align_blocks=0, msa_warps=0, streams=0):
    opts.driver = capi.CG_DRIVER_BATCHED
    opts.batch_anchors = batch
    opts.align_blocks = align_blocks
    opts.msa_warps = msa_warps
    opts.streams = streams
    return opts


def same(a, b, lens):
    fa, sa = a
    fb, sb = b
    assert np.array_equal(fa, fb), f"{int((fa != fb).sum())} anchors differ in flags"
    idx = np.nonzero(fa & capi.CG_RESULT_CORRECTED)[0]
    bad = [int(i) for i in idx if not np.array_equal(sa[i, :lens[i]], sb[i, :lens[i]])]
    assert not bad, f"{len(bad)} corrected anchors differ, first {bad[:5]}"


def small_reads(seed=43, n=12_000, **kw):
    cfg = sim.SimConfig(seed=seed, genome_length=60_000, repeat_families=3, repeat_copies=3, num_reads=n,
                        sub_rate_5p=0.002, sub_rate_3p=0.02, **kw)
    return sim.SimReads(cfg)


# shapes: (batch, persistent alignment blocks, MSA warps per block, pipelines)
SHAPES = [(2048, 7, 1, 1), (4096, 300, 3, 2), (1000, 1, 8, 2), (5000, 152, 2, 1)]


@pytest.mark.parametrize("shape", SHAPES)
def test_batched_matches_plain_across_shapes(shape):
    r = small_reads()
    (plain,), pst = run(capi.CareOptions.defaults(30.0), r)
    (bat,), bst = run(batched(capi.CareOptions.defaults(30.0), *shape), r)
    same(plain, bat, r.lengths)
    for k in COUNTERS:
        assert pst[k] == bst[k], k
    assert bst["graph_replays"] == r.n // shape[0]


@pytest.mark.parametrize("name", fx.case_names())
def test_batched_matches_reference_fixture(name):
    e = fx.manifest()[name]
    r = fx.reads_for(e)
    q = bool(e["options"].get("quality"))
    opts = batched(fx.options_for(e), 2048, 0, 4, 2)
    (res,), _ = run(opts, r, quality=q, forest=fx.forest_bytes(e))
    out = capi.apply_corrections(r.sequences, r.offsets, res[0], res[1])
    exp = fx.expected_output(name, r)
    bad = np.nonzero(out != exp)[0]
    assert bad.size == 0, f"{bad.size} bases differ from the reference output"


def test_batched_sub_range_with_remainder_and_repeated_calls():
    r = small_reads(seed=44)
    first, count = 1234, 9000  # 2 full batches of 4000 + a remainder of 1000
    (plain,), _ = run(capi.CareOptions.defaults(30.0), r, first=first, count=count)
    res, st = run(batched(capi.CareOptions.defaults(30.0), 4000, 0, 2, 2), r, first=first, count=count, repeat=2)
    same(plain, res[0], r.lengths[first:first + count])
    same(plain, res[1], r.lengths[first:first + count])
    assert st["graph_replays"] == 4


def test_batched_range_smaller_than_one_batch():
    # fewer anchors than a batch: everything runs as the remainder
    r = small_reads(seed=47, n=6_000)
    (plain,), _ = run(capi.CareOptions.defaults(30.0), r)
    (bat,), st = run(batched(capi.CareOptions.defaults(30.0), 0), r)
    same(plain, bat, r.lengths)
    assert st["graph_replays"] == 0


def test_batched_paired_end():
    cfg = sim.SimConfig(seed=45, genome_length=50_000, num_reads=10_000, paired=True, insert_mean=300,
                        insert_sd=30, sub_rate_5p=0.01, sub_rate_3p=0.01)
    r = sim.SimReads(cfg)
    o = capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE)
    (plain,), _ = run(o, r)
    o2 = batched(capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE), 2001, 0, 2, 2)  # rounded up to even
    (bat,), st = run(o2, r)
    same(plain, bat, r.lengths)
    assert st["batch_anchors"] == 2002


def test_batched_variable_lengths_and_quality():
    r = small_reads(seed=46, read_len_min=50, read_len_max=250)
    (plain,), _ = run(capi.CareOptions.defaults(30.0, use_quality_scores=1), r, quality=True)
    (bat,), _ = run(batched(capi.CareOptions.defaults(30.0, use_quality_scores=1), 3000, 0, 4, 2), r, quality=True)
    same(plain, bat, r.lengths)


def test_batched_autotuned_matches_plain():
    # large enough for the autotuner (at least two batches of 32768 in the sample)
    cfg = sim.scaled("c1_10mbp_repeats_se", genome_length=2_000_000)
    r = sim.SimReads(cfg)
    (plain,), pst = run(capi.CareOptions.defaults(30.0), r)
    (bat,), bst = run(batched(capi.CareOptions.defaults(30.0), 0), r)
    same(plain, bat, r.lengths)
    for k in COUNTERS:
        assert pst[k] == bst[k], k
    assert bst["batch_anchors"] in (32768, 65536, 131072)
    assert bst["streams"] in (1, 2)
    assert 1 <= bst["msa_warps"] <= 8
    assert bst["seconds_tune"] > 0


def test_batched_rejects_bad_shapes():
    for kw in ({"msa_warps": 9}, {"streams": 3}, {"align_blocks": -1}):
        o = capi.CareOptions.defaults(30.0, driver=capi.CG_DRIVER_BATCHED, **kw)
        with pytest.raises(capi.CareError):
            capi.CareGpu(o)
