"""File to file through the host layer (cg_correct_files = care::performCorrection).

The reference's own output FASTQ files were recorded (md5 of the whole file)
when the fixtures were made; the GPU engine's output files must be
byte-identical: same records, headers, qualities, and the same edit rules for
reads with and without ambiguous bases.
"""
import hashlib
import os

import pytest

import fixtures as fx
from rabbitqcplus_gb300 import capi

pytestmark = pytest.mark.gpu

FILE_CASES = [n for n in fx.case_names() if "output_file_md5" in fx.manifest()[n] and
              not fx.manifest()[n]["options"].get("forest")]


def md5_file(path):
    with open(path, "rb") as f:
        return hashlib.md5(f.read()).hexdigest()


@pytest.mark.parametrize("name", FILE_CASES)
def test_output_files_identical_to_reference(name, tmp_path):
    e = fx.manifest()[name]
    r = fx.reads_for(e)
    paired = bool(e["options"].get("paired"))
    if paired:
        ins = [str(tmp_path / "in_1.fq"), str(tmp_path / "in_2.fq")]
        r.write_fastq(ins[0], ins[1])
    else:
        ins = [str(tmp_path / "in.fq")]
        r.write_fastq(ins[0])
    assert [md5_file(p) for p in ins] == e["input_file_md5"]
    outs = [f"out_{i}.fq" for i in range(len(ins))]
    n = capi.correct_files(fx.options_for(e), ins, str(tmp_path), outs)
    assert n > 0
    got = [md5_file(os.path.join(tmp_path, o)) for o in outs]
    assert got == e["output_file_md5"]


LABEL_CASES = [n for n in fx.case_names() if "labels_file_md5" in fx.manifest()[n] and
               not fx.manifest()[n]["options"].get("forest")]


@pytest.mark.parametrize("host", [False, True], ids=["device_io", "host_io"])
@pytest.mark.parametrize("name", LABEL_CASES)
def test_labelled_output_files_identical_to_reference(name, host, tmp_path):
    """" care:q=N" labels: 0 none, 1 LQ anchor only, 2 LQ confirmed by candidate
    corrections, 3 HQ; reads after the last correction record get no label."""
    e = fx.manifest()[name]
    r = fx.reads_for(e)
    if e["options"].get("paired"):
        ins = [str(tmp_path / "in_1.fq"), str(tmp_path / "in_2.fq")]
        r.write_fastq(ins[0], ins[1])
    else:
        ins = [str(tmp_path / "in.fq")]
        r.write_fastq(ins[0])
    outs = [f"out_{i}.fq" for i in range(len(ins))]
    opts = fx.options_for(e)
    opts.host_file_io = int(host)
    capi.correct_files(opts, ins, str(tmp_path), outs, quality_labels=True)
    got = [md5_file(os.path.join(tmp_path, o)) for o in outs]
    assert got == e["labels_file_md5"]
