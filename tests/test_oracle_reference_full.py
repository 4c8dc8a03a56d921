"""The oracle against the reference's own build on whole workloads (no GPU).

Where the reference source tree exists, oracle/ref.mk compiles the
reference's CARE sources into oracle/_ref/ref_care; both correct every read of
a generated workload and the corrected outputs must be byte-identical.  The
200k-read workload runs by default (about half a minute on 8 threads); the
2M-read workload with repeats takes a few minutes and runs when
CARE_FULL_PARITY=1.
"""
import os

import pytest

import oracle
from oracle import port_speed


@pytest.fixture(scope="module")
def reference_build():
    if not os.path.isdir(os.path.join(oracle.reference_dir(), "src")):
        pytest.skip("reference source tree not present")
    assert oracle.build_reference()


@pytest.mark.slow
@pytest.mark.parametrize("config", [
    "c0_1mbp_se",
    pytest.param("c1_10mbp_repeats_se", marks=pytest.mark.skipif(os.environ.get("CARE_FULL_PARITY") != "1",
                                                                 reason="set CARE_FULL_PARITY=1")),
])
def test_oracle_output_identical_to_reference_build(reference_build, config):
    r = port_speed.compare(config, min(os.cpu_count() or 1, 8))
    assert r["outputs_identical"], r
