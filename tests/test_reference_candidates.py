"""Candidate correction does not depend on the order in which anchors run.

The reference saves candidate records under unsynchronised per-read flags
(include/corrector.hpp:1678-1681), so which records it saves depends on the
OpenMP schedule; the combine step (src/correctionresultoutput.cpp:1256-1551)
only reads records that the flags never drop, so the output does not.  The
GPU path relies on that: these tests check it on the reference itself (built
by oracle/ref.mk; skipped where it is absent) and on the oracle.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import fixtures as fx
import oracle

REF = os.path.join(fx.REPO, "oracle", "_ref", "ref_care")


def test_oracle_candidates_independent_of_thread_count():
    e = fx.manifest()["se_candidates"]
    r = fx.reads_for(e)
    runs = [oracle.Oracle(fx.options_for(e), r.sequences, r.offsets, None, threads=t).correct() for t in (1, 4)]
    (f1, s1, c1), (f4, s4, c4) = runs
    assert np.array_equal(f1, f4) and np.array_equal(s1, s4) and np.array_equal(c1, c4)


@pytest.mark.skipif(not os.path.exists(REF), reason="reference not built here")
def test_reference_candidate_output_independent_of_thread_count(tmp_path):
    e = fx.manifest()["se_candidates"]
    r = fx.reads_for(e)
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    digests = []
    for t in (1, 8):
        d = tmp_path / f"t{t}"
        d.mkdir()
        cmd = [REF, "-d", str(d), "-c", "30", "-k", "20", "-h", "48", "-t", str(t), "-i", fq, "-o", "out.fq",
               "--candidates", "--labels"]
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert p.returncode == 0, p.stdout[-2000:]
        with open(d / "out.fq", "rb") as f:
            digests.append(hashlib.md5(f.read()).hexdigest())
    assert digests[0] == digests[1] == e["labels_file_md5"][0]
