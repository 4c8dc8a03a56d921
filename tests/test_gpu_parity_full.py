"""Full-size parity: the CUDA path against the oracle on the measured workloads.

Every anchor of the 2M-read workloads (150 bp with repeats and a 5'->3'
rising error; variable length 50-250 bp), and a 200,000-anchor slice from
the middle of the 20M-read paired-end workload and of the 100M-read,
500 Mbp workload (every anchor of the slice, against tables of the whole read
set).  Both drivers, bit-exact: identical flags, identical corrected bases,
identical stage counters.  These are the sizes at which the alignment's
length tiers, the word-count grouping, the MSA refinement by subtraction and
the large-table candidate pass run most; the oracle itself is pinned to the
reference's own output (tests/test_oracle_golden.py).

The oracle builds its tables once per test on all host cores.
"""
import numpy as np
import pytest

import oracle
from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu

COUNTERS = (("raw_candidate_ids", 0), ("unique_candidates", 1), ("aligned_candidates", 2),
            ("msa_candidates", 3), ("corrected_anchors", 5), ("hq_anchors", 6))


def check(lengths, flags, seqs, oflags, oseqs, what):
    assert np.array_equal(flags, oflags), f"{what}: {int((flags != oflags).sum())} anchors differ in flags"
    idx = np.nonzero(flags & capi.CG_RESULT_CORRECTED)[0]
    mask = np.arange(seqs.shape[1])[None, :] < lengths[idx][:, None]
    a = np.where(mask, seqs[idx], 0)
    b = np.where(mask, oseqs[idx][:, :seqs.shape[1]], 0)
    bad = np.nonzero((a != b).any(axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} corrected anchors differ, first {idx[bad[:5]].tolist()}"


def gpu_run(reads, first, count, paired, driver):
    o = capi.CareOptions.defaults(30.0, driver=driver,
                                  pair_mode=capi.CG_PAIR_PE if paired else capi.CG_PAIR_SE)
    g = capi.CareGpu(o)
    g.append_reads(reads.sequences, reads.offsets)
    g.build_tables()
    flags, seqs = g.correct(first, count)
    st = g.stats()
    g.close()
    return flags, seqs, st


def run_config(cfg, first=0, count=None):
    r = sim.SimReads(cfg)
    count = r.n - first if count is None else count
    o = capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE if cfg.paired else capi.CG_PAIR_SE)
    orc = oracle.Oracle(o, r.sequences, r.offsets, None)
    oflags, oseqs, cnt = orc.correct(first, count)
    orc.close()
    lengths = r.lengths[first:first + count]
    for driver, name in ((capi.CG_DRIVER_PLAIN, "plain"), (capi.CG_DRIVER_BATCHED, "batched")):
        flags, seqs, st = gpu_run(r, first, count, cfg.paired, driver)
        check(lengths, flags, seqs, oflags, oseqs, name)
        for key, i in COUNTERS:
            assert st[key] == cnt[i], f"{name}: {key} {st[key]} != {cnt[i]}"
        del flags, seqs
    assert int((oflags & capi.CG_RESULT_CORRECTED).astype(bool).sum()) > count // 4


@pytest.mark.parametrize("name", ["c1_10mbp_repeats_se", "c3_10mbp_varlen"])
def test_every_anchor_of_2m_read_workload(name):
    run_config(sim.CONFIGS[name])


@pytest.mark.parametrize("name", ["c2_100mbp_pe", "c4_500mbp_se"])
def test_middle_slice_of_large_workload(name):
    cfg = sim.CONFIGS[name]
    first = (cfg.num_reads // 2) & ~1
    run_config(cfg, first, 200_000)
