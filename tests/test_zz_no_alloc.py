"""cg_get_candidates_noalloc: the candidate lookup that allocates no device memory.

It serves callers that cannot call cudaMalloc (an application that owns the
whole device budget, or a latency-sensitive per-read loop).  Its result must
equal cg_get_candidates' exactly (integer ids, so no tolerance), call after
call: the shared scratch array keeps the previous call's contents and the
entry point must clear what has to start at zero.  This file sorts last so a
failure here comes after every other test has run.
"""
import numpy as np
import pytest

from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu


def test_noalloc_candidates_equal_allocating_entry_point_on_consecutive_calls():
    cfg = sim.SimConfig(seed=61, genome_length=30_000, repeat_families=2, repeat_copies=3, num_reads=6_000,
                        sub_rate_5p=0.002, sub_rate_3p=0.02)
    r = sim.SimReads(cfg)
    g = capi.CareGpu(capi.CareOptions.defaults(30.0))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    out = np.zeros(8192, dtype=np.uint32)
    anchors = [0, 1, 2, 17, 999, 3000, 5999, 4242]
    for a in anchors:
        ref = g.candidates(a)
        # two calls in a row: the second must not see the first's leftovers
        for _ in range(2):
            out.fill(0xFFFFFFFF)
            n = g.candidates_noalloc(a, out)
            assert n == ref.size
            assert np.array_equal(out[:n], ref), f"anchor {a}"
    # a capacity below the count: the count is still reported, only capacity ids are written
    a = int(np.argmax([g.candidates(x).size for x in anchors]))
    full = g.candidates(anchors[a])
    small = np.zeros(max(1, full.size // 2), dtype=np.uint32)
    n = g.candidates_noalloc(anchors[a], small)
    assert n == full.size and np.array_equal(small, full[:small.size])
    g.close()


def with_copies(r, read, copies):
    """The read set plus `copies` exact copies of read `read` at its end."""
    s = r.sequences[r.offsets[read]:r.offsets[read + 1]]
    seqs = np.concatenate([r.sequences] + [s] * copies)
    offs = np.concatenate([r.offsets, r.offsets[-1] + len(s) * np.arange(1, copies + 1, dtype=np.uint64)])
    return seqs, offs.astype(np.uint64)


def raw_hits(g, anchor):
    before = g.stats()["raw_candidate_ids"]
    ids = g.candidates(anchor)
    return g.stats()["raw_candidate_ids"] - before, ids


def test_noalloc_large_buckets_and_rejection_above_its_limit():
    cfg = sim.SimConfig(seed=62, genome_length=30_000, num_reads=6_000)
    r = sim.SimReads(cfg)
    out = np.zeros(16384, dtype=np.uint32)
    # 60 copies of one read: every map's bucket of the copies holds 60 ids, so an
    # anchor among them has more than 1024 raw hits (the single-pass large-table
    # gather here, the split pass in cg_get_candidates)
    seqs, offs = with_copies(r, 5, 60)
    g = capi.CareGpu(capi.CareOptions.defaults(30.0))
    g.append_reads(seqs, offs)
    g.build_tables()
    a = r.n + 3
    raw, ref = raw_hits(g, a)
    assert raw > 1024, raw
    for _ in range(2):
        out.fill(0xFFFFFFFF)
        n = g.candidates_noalloc(a, out)
        assert n == ref.size and np.array_equal(out[:n], ref)
    g.close()
    # 250 copies at coverage 200 (buckets of up to 500 ids): more than the 8192
    # raw hits the scratch array holds -> CG_ERR_INVALID_ARGUMENT, and the next
    # call within the limit still equals cg_get_candidates
    seqs, offs = with_copies(r, 5, 250)
    g = capi.CareGpu(capi.CareOptions.defaults(200.0))
    g.append_reads(seqs, offs)
    g.build_tables()
    a = r.n + 7
    raw, ref = raw_hits(g, a)
    assert raw > 8192, raw
    with pytest.raises(capi.CareError, match="invalid argument"):
        g.candidates_noalloc(a, out)
    for b in (17, 4000):
        raw_b, ref_b = raw_hits(g, b)
        assert raw_b <= 8192
        out.fill(0xFFFFFFFF)
        n = g.candidates_noalloc(b, out)
        assert n == ref_b.size and np.array_equal(out[:n], ref_b), f"anchor {b}"
    g.close()
