"""GPU parity: the CUDA path against the reference's fixtures and the oracle.

All calls go through the C ABI (libcaregpu.so via ctypes).  Integer and
order-fixed float work, so the bar is bit-exact: identical flags and
identical corrected bases for every anchor.
"""
import os

import numpy as np
import pytest

import fixtures as fx
import oracle
from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu


def run_gpu(opts, reads, quality=False, batch=0, forest=None):
    opts.batch_anchors = batch
    g = capi.CareGpu(opts)
    g.append_reads(reads.sequences, reads.offsets, reads.qualities if quality else None)
    g.build_tables()
    if forest:
        g.load_forest(forest)
    flags, seqs = g.correct()
    stats = g.stats()
    return g, flags, seqs, stats


def assert_same_results(reads, flags, seqs, oflags, oseqs):
    assert np.array_equal(flags, oflags), f"{int((flags != oflags).sum())} anchors differ in flags"
    idx = np.nonzero(flags & capi.CG_RESULT_CORRECTED)[0]
    lens = reads.lengths
    bad = [int(i) for i in idx if not np.array_equal(seqs[i, :lens[i]], oseqs[i, :lens[i]])]
    assert not bad, f"{len(bad)} corrected anchors differ, first {bad[:5]}"


@pytest.mark.parametrize("name", fx.case_names())
def test_gpu_matches_reference_fixture(name):
    e = fx.manifest()[name]
    r = fx.reads_for(e)
    q = bool(e["options"].get("quality"))
    g, flags, seqs, _ = run_gpu(fx.options_for(e), r, quality=q, forest=fx.forest_bytes(e))
    out = capi.apply_corrections(r.sequences, r.offsets, flags, seqs)
    exp = fx.expected_output(name, r)
    bad = np.nonzero(out != exp)[0]
    assert bad.size == 0, f"{bad.size} bases differ from the reference output"
    assert r.score(out) == e["score"]
    g.close()


STAGE_CASES = [n for n in fx.case_names() if fx.manifest()[n].get("stage_anchors")]


@pytest.mark.parametrize("name", STAGE_CASES)
def test_gpu_signatures_and_candidates_match_reference_stages(name):
    e = fx.manifest()[name]
    r = fx.reads_for(e)
    q = bool(e["options"].get("quality"))
    g, _, _, st = run_gpu(fx.options_for(e), r, quality=q)
    stages = fx.load_stages(name)
    ids = sorted(stages["sigs"])
    sig = g.signatures(0, len(ids), st["num_maps"])
    for i in ids:
        assert sig[i].tolist() == stages["sigs"][i], f"signature of read {i}"
    for a in stages["anchors"]:
        assert g.candidates(a["id"]).tolist() == a["cand"], f"candidates of anchor {a['id']}"
    g.close()


@pytest.mark.parametrize("batch", [0, 1, 7, 1000])
def test_gpu_matches_oracle_across_batch_sizes(batch):
    cfg = sim.SimConfig(seed=41, genome_length=40_000, repeat_families=3, repeat_copies=3, num_reads=8_000,
                        sub_rate_5p=0.002, sub_rate_3p=0.02)
    r = sim.SimReads(cfg)
    opts = capi.CareOptions.defaults(30.0)
    g, flags, seqs, _ = run_gpu(opts, r, batch=batch)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None)
    oflags, oseqs, _ = orc.correct()
    assert_same_results(r, flags, seqs, oflags, oseqs)
    g.close()


def test_gpu_matches_oracle_c0_shape_full_size():
    """1 Mbp genome, 200k x 150 bp reads at 30x, 1% substitutions: every anchor."""
    r = sim.SimReads(sim.CONFIGS["c0_1mbp_se"])
    opts = capi.CareOptions.defaults(30.0)
    g, flags, seqs, st = run_gpu(opts, r)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None)
    oflags, oseqs, cnt = orc.correct()
    assert_same_results(r, flags, seqs, oflags, oseqs)
    # the device counters agree with the oracle's
    assert st["raw_candidate_ids"] == cnt[0]
    assert st["unique_candidates"] == cnt[1]
    assert st["aligned_candidates"] == cnt[2]
    assert st["msa_candidates"] == cnt[3]
    assert st["corrected_anchors"] == cnt[5]
    assert st["hq_anchors"] == cnt[6]
    g.close()


def test_gpu_matches_oracle_repeats_sample():
    """c1 shape (repeats, rising 5'->3' error) at 2 Mbp, 400k reads: a sample of anchors."""
    cfg = sim.scaled("c1_10mbp_repeats_se", 2_000_000)
    r = sim.SimReads(cfg)
    opts = capi.CareOptions.defaults(30.0)
    g, flags, seqs, _ = run_gpu(opts, r)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None)
    first, count = 100_000, 40_000
    oflags, oseqs, _ = orc.correct(first, count)
    sub = sim.SimReads.__new__(sim.SimReads)
    sub.lengths = r.lengths[first:first + count]
    assert_same_results(sub, flags[first:first + count], seqs[first:first + count], oflags, oseqs)
    g.close()


def test_gpu_paired_end_matches_oracle():
    cfg = sim.SimConfig(seed=43, genome_length=60_000, num_reads=12_000, paired=True, repeat_families=3,
                        repeat_copies=3)
    r = sim.SimReads(cfg)
    opts = capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE)
    g, flags, seqs, _ = run_gpu(opts, r, batch=1000)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE), r.sequences, r.offsets, None)
    oflags, oseqs, _ = orc.correct()
    assert_same_results(r, flags, seqs, oflags, oseqs)
    g.close()


@pytest.mark.parametrize("forest_file", ["forest_anchor.bin", "forest_varlen.bin"])
def test_gpu_forest_matches_oracle_with_quality_and_tree_limit(forest_file):
    """The fixture forest (16 trees) and the workload forest the learned
    decision is compared with (64 trees of up to 1024 leaves)."""
    with open(os.path.join(fx.GOLDEN, forest_file), "rb") as f:
        forest = f.read()
    cfg = sim.SimConfig(seed=45, genome_length=40_000, num_reads=8_000, repeat_families=3, repeat_copies=3,
                        read_len_min=100, read_len_max=150, sub_rate_5p=0.004, sub_rate_3p=0.03)
    r = sim.SimReads(cfg)
    for q, trees in ((0, 0), (1, 5)):
        kw = dict(use_quality_scores=q, correction_type=capi.CG_CORR_FOREST, threshold_anchor=0.6)
        opts = capi.CareOptions.defaults(30.0, **kw)
        opts.batch_anchors = 0
        g = capi.CareGpu(opts)
        g.append_reads(r.sequences, r.offsets, r.qualities if q else None)
        g.build_tables()
        g.load_forest(forest, trees)
        flags, seqs = g.correct()
        orc = oracle.Oracle(capi.CareOptions.defaults(30.0, **kw), r.sequences, r.offsets, r.qualities if q else None)
        orc.load_forest(forest, trees if trees else 0xFFFFFFFF, 0.6)
        oflags, oseqs, _ = orc.correct()
        assert_same_results(r, flags, seqs, oflags, oseqs)
        g.close()


def test_gpu_quality_scores_match_oracle():
    cfg = sim.SimConfig(seed=44, genome_length=40_000, num_reads=8_000, repeat_families=2, repeat_copies=3)
    r = sim.SimReads(cfg)
    opts = capi.CareOptions.defaults(30.0, use_quality_scores=1)
    g, flags, seqs, _ = run_gpu(opts, r, quality=True)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0, use_quality_scores=1), r.sequences, r.offsets, r.qualities)
    oflags, oseqs, _ = orc.correct()
    assert_same_results(r, flags, seqs, oflags, oseqs)
    g.close()


def test_gpu_edge_cases_short_reads_and_ambiguous():
    """Reads shorter than k, reads with N, a read of length 1, duplicate reads."""
    rng = np.random.default_rng(3)
    genome = rng.choice(np.frombuffer(b"ACGT", np.uint8), 3000)
    seqs, offs = [], [0]
    for i in range(1200):
        L = int(rng.integers(1, 40)) if i % 50 == 0 else 100
        s = int(rng.integers(0, len(genome) - L))
        read = genome[s:s + L].copy()
        if i % 37 == 0:
            read[int(rng.integers(0, L))] = ord("N")
        if i % 41 == 0:
            read[int(rng.integers(0, L))] = ord("a")
        seqs.append(read)
        offs.append(offs[-1] + L)
    seqs.append(seqs[10].copy())  # an exact duplicate
    offs.append(offs[-1] + len(seqs[-1]))
    allseq = np.concatenate(seqs)
    offs = np.array(offs, dtype=np.uint64)
    for excl in (0, 1):
        opts = capi.CareOptions.defaults(30.0, exclude_ambiguous_reads=excl)
        g = capi.CareGpu(opts)
        g.append_reads(allseq, offs)
        g.build_tables()
        flags, out = g.correct()
        orc = oracle.Oracle(capi.CareOptions.defaults(30.0, exclude_ambiguous_reads=excl), allseq, offs, None)
        oflags, oseqs, _ = orc.correct()
        r = sim.SimReads.__new__(sim.SimReads)
        r.lengths = np.diff(offs).astype(np.int32)
        assert_same_results(r, flags, out, oflags, oseqs)
        g.close()


def test_gpu_rejects_bad_arguments():
    opts = capi.CareOptions.defaults(30.0)
    g = capi.CareGpu(opts)
    with pytest.raises(capi.CareError):
        g.build_tables()  # no reads yet
    seq = np.frombuffer(b"ACGT" * 100, np.uint8)
    g.append_reads(seq, np.array([0, 200, 400], np.uint64))
    g.build_tables()
    with pytest.raises(capi.CareError):
        g.correct(1, 5)  # out of range
    with pytest.raises(capi.CareError):
        g.append_reads(seq, np.array([0, 400], np.uint64))  # after build
    g.close()
    bad = capi.CareOptions.defaults(30.0, correction_type=capi.CG_CORR_PRINT)
    with pytest.raises(capi.CareError):
        capi.CareGpu(bad)
    bad = capi.CareOptions.defaults(30.0, num_hash_functions=49)
    with pytest.raises(capi.CareError):
        capi.CareGpu(bad)
