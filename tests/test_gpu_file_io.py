"""The device file path (FASTQ parsing and output records on the GPU) writes
the same files as the host reader and writer.

cg_correct_files parses plain 4-line FASTQ input and writes the output
records on the device; `host_file_io = 1` forces the host path.  Both must give
byte-identical files for single-end and paired-end input, with and without
quality labels, from plain and gzip input; input the device path does not take
(CRLF line ends) must still give the same records through the host path.
"""
import gzip
import hashlib
import os
import shutil

import pytest

from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu


def md5(path):
    with open(path, "rb") as f:
        return hashlib.md5(f.read()).hexdigest()


def run(opts, ins, outdir, nout, labels=False, host=False, gz_out=False):
    opts.host_file_io = 1 if host else 0
    os.makedirs(outdir, exist_ok=True)
    outs = [f"out_{i}.fq" + (".gz" if gz_out else "") for i in range(nout)]
    n = capi.correct_files(opts, ins, str(outdir), outs, quality_labels=labels, gz_output=gz_out)
    return n, [os.path.join(outdir, o) for o in outs]


def se_reads(seed=51):
    return sim.SimReads(sim.SimConfig(seed=seed, genome_length=60_000, repeat_families=3, repeat_copies=3,
                                      num_reads=12_000, n_read_fraction=0.02, sub_rate_5p=0.002, sub_rate_3p=0.02))


@pytest.mark.parametrize("labels", [False, True])
def test_single_end_device_and_host_files_identical(tmp_path, labels):
    r = se_reads()
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    o = capi.CareOptions.defaults(30.0, driver=capi.CG_DRIVER_BATCHED)
    nd, dev = run(o, [fq], tmp_path / "dev", 1, labels)
    nh, host = run(capi.CareOptions.defaults(30.0), [fq], tmp_path / "host", 1, labels, host=True)
    assert nd == nh > 0
    assert md5(dev[0]) == md5(host[0])


def test_paired_end_two_files_and_quality_scores(tmp_path):
    r = sim.SimReads(sim.SimConfig(seed=52, genome_length=50_000, num_reads=10_000, paired=True,
                                   sub_rate_5p=0.01, sub_rate_3p=0.01, indel_rate=0.0001))
    ins = [str(tmp_path / "in_1.fq"), str(tmp_path / "in_2.fq")]
    r.write_fastq(ins[0], ins[1])
    mk = lambda: capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE, use_quality_scores=1)
    nd, dev = run(mk(), ins, tmp_path / "dev", 2)
    nh, host = run(mk(), ins, tmp_path / "host", 2, host=True)
    assert nd == nh > 0
    assert [md5(p) for p in dev] == [md5(p) for p in host]
    # one output file: both mates interleaved in read order
    nd1, dev1 = run(mk(), ins, tmp_path / "dev1", 1)
    nh1, host1 = run(mk(), ins, tmp_path / "host1", 1, host=True)
    assert md5(dev1[0]) == md5(host1[0])


def test_gzip_input_and_output(tmp_path):
    r = se_reads(53)
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    with open(fq, "rb") as a, gzip.open(str(tmp_path / "in.fq.gz"), "wb") as b:
        shutil.copyfileobj(a, b)
    nd, dev = run(capi.CareOptions.defaults(30.0), [str(tmp_path / "in.fq.gz")], tmp_path / "dev", 1, gz_out=True)
    nh, host = run(capi.CareOptions.defaults(30.0), [fq], tmp_path / "host", 1, host=True)
    assert nd == nh
    with gzip.open(dev[0], "rb") as f:
        assert hashlib.md5(f.read()).hexdigest() == md5(host[0])


def test_input_the_device_path_does_not_take(tmp_path):
    r = se_reads(54)
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    crlf = str(tmp_path / "crlf.fq")
    with open(fq, "rb") as a, open(crlf, "wb") as b:
        b.write(a.read().replace(b"\n", b"\r\n"))
    nd, dev = run(capi.CareOptions.defaults(30.0), [crlf], tmp_path / "dev", 1)  # falls back to the host path
    nh, host = run(capi.CareOptions.defaults(30.0), [fq], tmp_path / "host", 1, host=True)
    assert nd == nh
    assert md5(dev[0]) == md5(host[0])


@pytest.mark.parametrize("paired", [False, True])
def test_large_input_corrected_and_written_range_by_range(tmp_path, paired):
    # more than 262144 reads: the device path corrects and writes the output in
    # several ranges (the writer thread writes one while the next is corrected)
    cfg = sim.SimConfig(seed=54, genome_length=400_000, num_reads=600_000, paired=paired, sub_rate_5p=0.002,
                        sub_rate_3p=0.02)
    r = sim.SimReads(cfg)
    if paired:
        ins = [str(tmp_path / "in_1.fq"), str(tmp_path / "in_2.fq")]
        r.write_fastq(ins[0], ins[1])
        mk = lambda: capi.CareOptions.defaults(30.0, pair_mode=capi.CG_PAIR_PE, driver=capi.CG_DRIVER_BATCHED)
        nout = 2
    else:
        ins = [str(tmp_path / "in.fq")]
        r.write_fastq(ins[0])
        mk = lambda: capi.CareOptions.defaults(30.0, driver=capi.CG_DRIVER_BATCHED)
        nout = 1
    nd, dev = run(mk(), ins, tmp_path / "dev", nout, labels=True)
    nh, host = run(mk(), ins, tmp_path / "host", nout, labels=True, host=True)
    assert nd == nh > 0
    assert [md5(p) for p in dev] == [md5(p) for p in host]
