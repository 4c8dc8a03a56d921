"""The device alignment's orientation shortcut, checked on the CPU.

align_lane_kernel scans each candidate's predicted orientation in full and
the other one only where a one-plane test of all its shifts cannot rule out a
tie; where it rules it out, it writes the first orientation's result as the
reference's choice.  This checks that claim against the oracle's full
two-orientation alignment and the reference's orientation rule, for every
candidate of a sample of anchors and for either orientation scanned first
(the prediction only decides which one that is): no decided case may differ.
The GPU parity tests show the kernel's output equal to the oracle's; this
shows the rule it relies on holds case by case, including where the
prediction is wrong.
"""
import pytest

import oracle
from rabbitqcplus_gb300 import capi, sim

# workload, and the smallest share of cases the shortcut must decide
CASES = {
    # 150 bp reads, 2% diverged repeats, rising 3' error: about half
    "repeats": (sim.SimConfig(seed=91, genome_length=300_000, repeat_families=6, repeat_copies=4,
                              num_reads=60_000, sub_rate_5p=0.002, sub_rate_3p=0.02), 0.3),
    # 50-250 bp reads: short anchors (minimum overlap under 32) never take the
    # shortcut, nor do the pairs whose shorter read is short
    "varlen": (sim.SimConfig(seed=92, genome_length=300_000, repeat_families=6, repeat_copies=4,
                             num_reads=60_000, read_len_min=50, read_len_max=250,
                             sub_rate_5p=0.002, sub_rate_3p=0.02), 0.15),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_shortcut_never_changes_the_orientation(name):
    cfg, share = CASES[name]
    r = sim.SimReads(cfg)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None)
    res = orc.check_orientation_shortcut(r.n // 3, 6000)
    orc.close()
    assert res["wrong"] == 0, res
    # a candidate with one orientation that is chosen on its own and rules the
    # other out is decided when that orientation is scanned first
    assert res["decided"] > share * res["cases"], res
