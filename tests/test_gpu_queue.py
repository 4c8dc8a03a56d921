"""The queue protocol of the host layer (performCorrectionOutToQueue, through
its sink form): 1 MiB chunks of whole records whose concatenation is the
output file, the same from the device file path (chunks copied from device
memory straight into the consumer's buffers) and the host path.

tests/queue_driver.cpp is compiled against the library here (g++).
"""
import hashlib
import os
import shutil
import subprocess

import pytest

from rabbitqcplus_gb300 import _lib, capi, sim

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    lib = _lib.build_gpu()
    exe = str(tmp_path_factory.mktemp("qd") / "queue_driver")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"),
                    "-I", os.path.join(REPO, "rabbitqcplus_gb300", "csrc", "host"),
                    os.path.join(HERE, "queue_driver.cpp"), "-o", exe, "-L", libdir, "-lcaregpu",
                    "-Wl,-rpath," + libdir], check=True)
    return exe


def md5(path):
    with open(path, "rb") as f:
        return hashlib.md5(f.read()).hexdigest()


def run_driver(exe, mode, pe, prefix, ins):
    r = subprocess.run([exe, mode, "pe" if pe else "se", prefix, *ins], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    f = r.stdout.split()
    return {f[i]: int(f[i + 1]) for i in range(0, len(f), 2)}


@pytest.mark.parametrize("pe", [False, True])
def test_queue_chunks_equal_the_output_files(driver, tmp_path, pe):
    if pe:
        r = sim.SimReads(sim.SimConfig(seed=61, genome_length=200_000, num_reads=40_000, paired=True))
        ins = [str(tmp_path / "in_1.fq"), str(tmp_path / "in_2.fq")]
        r.write_fastq(ins[0], ins[1])
    else:
        r = sim.SimReads(sim.SimConfig(seed=62, genome_length=200_000, num_reads=40_000, n_read_fraction=0.01))
        ins = [str(tmp_path / "in.fq")]
        r.write_fastq(ins[0])
    dev = run_driver(driver, "device", pe, str(tmp_path / "qdev_"), ins)
    host = run_driver(driver, "host", pe, str(tmp_path / "qhost_"), ins)
    assert dev["device"] == 1 and host["device"] == 0
    assert dev["records"] == host["records"] > 0
    assert dev["chunks"] > 1  # 40k reads of ~330 bytes span several 1 MiB chunks
    assert dev["chunks"] == host["chunks"]  # the same cut points
    o = capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE if pe else capi.CG_PAIR_SE)
    outs = [f"out_{i}.fq" for i in range(len(ins))]
    capi.correct_files(o, ins, str(tmp_path), outs)
    for i, name in enumerate(outs):
        want = md5(tmp_path / name)
        assert md5(tmp_path / f"qdev_{i}.fq") == want
        assert md5(tmp_path / f"qhost_{i}.fq") == want
