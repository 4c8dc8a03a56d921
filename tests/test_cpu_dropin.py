"""The drop-in shim inside RabbitQCPlus's own caller (no GPU needed).

Where the reference source tree exists ($CARE_REFERENCE_DIR, or `reference`
beside this repository), oracle/ref.mk builds care_gpu_dropin: RabbitQCPlus's
main_correction (src/main_correct_cpu.cpp) and CARE objects with
dispatch_care_correct_cpu.o replaced by
rabbitqcplus_gb300/csrc/host/dispatch_care_correct_gpu.cpp, linked against
libcaregpu.so, driven by tests/shim_consumer.cpp the way SeQc::careProcess and
FileReader::Read drive the reference (the moodycamel queue protocol).  The
test checks that it compiles and links against the reference's headers, that
every forwarded care::ProgramOptions field reaches the GB300 options, and that
a run goes through the reference's option parsing into the shim: without a
GPU the engine's error comes back to the consumer as an exception (exit 3);
with one, the queue carries the corrected records.
"""
import os
import subprocess

import pytest

import oracle
from rabbitqcplus_gb300 import _lib, sim

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin():
    ref = oracle.reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("reference source tree not present")
    _lib.build_gpu()
    r = subprocess.run(["make", "-f", os.path.join("oracle", "ref.mk"), f"REF={ref}", "-j8", "dropin"], cwd=REPO,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    return os.path.join(REPO, "oracle", "_ref", "care_gpu_dropin")


def test_every_forwarded_option_reaches_the_engine(dropin):
    r = subprocess.run([dropin, "--mapping"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0 and "mapping ok" in r.stdout, r.stdout


def test_rabbitqcplus_caller_runs_through_the_shim(dropin, tmp_path):
    reads = sim.SimReads(sim.SimConfig(seed=3, genome_length=20_000, num_reads=4_000))
    fq = str(tmp_path / "in.fq")
    reads.write_fastq(fq)
    r = subprocess.run([dropin, "--queue", "4", fq, str(tmp_path / "out.fq")], cwd=str(tmp_path),
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
    # main_correction parsed the options and handed them to the shim
    assert "CARE CORRECT CPU will be started" in r.stderr
    if r.returncode == 3:
        assert r.stdout.startswith("error: ") and "CUDA" in r.stdout, r.stdout
    else:
        assert r.returncode == 0, r.stdout + r.stderr[-2000:]
        assert r.stdout.startswith("changNum "), r.stdout
        assert os.path.getsize(str(tmp_path / "out.fq")) > 0
