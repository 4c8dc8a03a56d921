"""Generate the parity fixtures in tests/golden/ by running the reference.

Run from the repository root, in a container where the reference tree exists:

    python tests/golden/make_golden.py [--ref PATH_TO_RABBITQCPLUS]

(default: $CARE_REFERENCE_DIR, else a `reference` directory beside this repository)

For every case in CASES it
  1. generates the seeded synthetic reads (rabbitqcplus_gb300.sim),
  2. writes them as FASTQ and runs the reference's own care::performCorrection
     (oracle/_ref/ref_care, compiled from the reference's sources by oracle/ref.mk),
  3. stores the reference's output as a compact diff against the input reads
     (<case>.npz: every differing position as read id (delta coded), position, base) plus the md5 of the
     full output sequences and of the generated input, in manifest.json.
It also dumps the reference's per-anchor intermediate results (signatures,
candidate lists, alignments, MSA consensus/support, correction) for the first
anchors of some cases with oracle/_ref/ref_stages (<case>.stages.txt.gz).

The fixtures are regenerated only by this script; tests read them and re-create
the inputs from the recorded generator configs.
"""
from __future__ import annotations

import argparse
import dataclasses
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from rabbitqcplus_gb300 import sim  # noqa: E402

# name -> (generator config, reference options, stage-dump anchors)
CASES = {
    "se_basic": (sim.SimConfig(seed=101, genome_length=50_000, num_reads=10_000),
                 {"coverage": 30, "k": 20}, 40),
    "se_repeats": (sim.SimConfig(seed=102, genome_length=60_000, repeat_families=6, repeat_copies=4,
                                 repeat_min_len=1000, repeat_max_len=3000, repeat_divergence=0.02,
                                 num_reads=12_000, sub_rate_5p=0.002, sub_rate_3p=0.02),
                   {"coverage": 30, "k": 20}, 60),
    "se_varlen": (sim.SimConfig(seed=103, genome_length=60_000, repeat_families=4, repeat_copies=4,
                                repeat_min_len=1000, repeat_max_len=3000, num_reads=12_000,
                                read_len_min=50, read_len_max=250, sub_rate_5p=0.002, sub_rate_3p=0.02),
                  {"coverage": 30, "k": 20}, 40),
    "se_quality": (sim.SimConfig(seed=104, genome_length=50_000, num_reads=10_000),
                   {"coverage": 30, "k": 20, "quality": True}, 40),
    "se_ambiguous": (sim.SimConfig(seed=105, genome_length=50_000, num_reads=10_000, n_read_fraction=0.03),
                     {"coverage": 30, "k": 20}, 0),
    "se_exclude_ambiguous": (sim.SimConfig(seed=106, genome_length=40_000, num_reads=8_000, n_read_fraction=0.05),
                             {"coverage": 30, "k": 20, "exclude_ambiguous": True}, 0),
    "se_k32_auto": (sim.SimConfig(seed=107, genome_length=50_000, num_reads=8_000, read_len_min=180,
                                  read_len_max=200),
                    {"coverage": 30, "k": 0}, 0),
    "se_cov20": (sim.SimConfig(seed=108, genome_length=60_000, repeat_families=4, repeat_copies=3,
                               num_reads=8_000, sub_rate_5p=0.01, sub_rate_3p=0.01),
                 {"coverage": 20, "k": 20}, 0),
    "pe_basic": (sim.SimConfig(seed=109, genome_length=50_000, num_reads=10_000, paired=True,
                               repeat_families=3, repeat_copies=3, indel_rate=0.0001),
                 {"coverage": 30, "k": 20, "paired": True}, 0),
    # reads shorter than the longest with quality scores: a reverse-complement
    # candidate's reversed quality row starts with the padding
    "se_varlen_quality": (sim.SimConfig(seed=114, genome_length=60_000, repeat_families=4, repeat_copies=4,
                                        num_reads=12_000, read_len_min=60, read_len_max=240, sub_rate_5p=0.002,
                                        sub_rate_3p=0.02),
                          {"coverage": 30, "k": 20, "quality": True}, 0),
    # reads longer than 256 bp (block-per-anchor kernels), k autodetected (32)
    "se_long_quality": (sim.SimConfig(seed=115, genome_length=60_000, repeat_families=4, repeat_copies=4,
                                      num_reads=5_000, read_len_min=180, read_len_max=400, sub_rate_5p=0.002,
                                      sub_rate_3p=0.02),
                        {"coverage": 25, "k": 0, "quality": True}, 0),
    "pe_quality_varlen": (sim.SimConfig(seed=116, genome_length=50_000, num_reads=10_000, paired=True,
                                        repeat_families=3, repeat_copies=3, read_len_min=100, read_len_max=150),
                          {"coverage": 25, "k": 20, "paired": True, "quality": True}, 0),
    # fewer maps and a shorter k
    "se_maps24_k16": (sim.SimConfig(seed=117, genome_length=50_000, num_reads=10_000, repeat_families=3,
                                    repeat_copies=3),
                      {"coverage": 30, "k": 16, "maps": 24}, 0),
    # candidate correction (--candidateCorrection) and the combine step
    "se_candidates": (sim.SimConfig(seed=110, genome_length=60_000, repeat_families=6, repeat_copies=4,
                                    repeat_min_len=1000, repeat_max_len=3000, repeat_divergence=0.02,
                                    num_reads=12_000, sub_rate_5p=0.002, sub_rate_3p=0.02),
                      {"coverage": 30, "k": 20, "candidates": True}, 0),
    "pe_candidates": (sim.SimConfig(seed=111, genome_length=50_000, num_reads=10_000, paired=True,
                                    repeat_families=3, repeat_copies=3),
                      {"coverage": 30, "k": 20, "paired": True, "candidates": True}, 0),
    "se_candidates_varlen_quality": (sim.SimConfig(seed=112, genome_length=60_000, repeat_families=4,
                                                   repeat_copies=4, num_reads=12_000, read_len_min=50,
                                                   read_len_max=250, sub_rate_5p=0.002, sub_rate_3p=0.02),
                                     {"coverage": 30, "k": 20, "quality": True, "candidates": True,
                                      "new_columns": 25}, 0),
    "se_long_candidates": (sim.SimConfig(seed=119, genome_length=60_000, repeat_families=4, repeat_copies=4,
                                         num_reads=5_000, read_len_min=200, read_len_max=380, sub_rate_5p=0.002,
                                         sub_rate_3p=0.02),
                           {"coverage": 25, "k": 0, "quality": True, "candidates": True}, 0),
    # the last three reads are ambiguous and excluded, so they have no record:
    # the reference writes no quality label for reads after the last record
    "se_label_tail": (sim.SimConfig(seed=118, genome_length=40_000, num_reads=8_000, n_read_fraction=0.3),
                      {"coverage": 30, "k": 20, "exclude_ambiguous": True}, 0),
    "se_candidates_tail": (sim.SimConfig(seed=118, genome_length=40_000, num_reads=8_000, n_read_fraction=0.3),
                           {"coverage": 30, "k": 20, "exclude_ambiguous": True, "candidates": True}, 0),
    # lossy quality store (--qualityScoreBits): binned scores; with reads of
    # several lengths a reverse-complement candidate's reversed row starts
    # with the first bin's score
    "se_quality_bits2": (sim.SimConfig(seed=120, genome_length=50_000, num_reads=10_000, repeat_families=3,
                                       repeat_copies=3, sub_rate_5p=0.004, sub_rate_3p=0.03),
                         {"coverage": 30, "k": 20, "quality": True, "quality_bits": 2}, 0),
    "se_varlen_quality_bits1": (sim.SimConfig(seed=121, genome_length=60_000, repeat_families=4, repeat_copies=4,
                                              num_reads=12_000, read_len_min=60, read_len_max=240,
                                              sub_rate_5p=0.004, sub_rate_3p=0.03),
                                {"coverage": 30, "k": 20, "quality": True, "quality_bits": 1}, 0),
    "pe_varlen_quality_bits2": (sim.SimConfig(seed=122, genome_length=50_000, num_reads=10_000, paired=True,
                                              repeat_families=3, repeat_copies=3, read_len_min=100,
                                              read_len_max=150),
                                {"coverage": 25, "k": 20, "paired": True, "quality": True, "quality_bits": 2}, 0),
    # --fixedNumberOfReads: only the first reads are corrected as anchors,
    # every read is a candidate
    "se_fixed_reads": (sim.SimConfig(seed=123, genome_length=50_000, num_reads=10_000, repeat_families=3,
                                     repeat_copies=3, sub_rate_5p=0.002, sub_rate_3p=0.02),
                       {"coverage": 30, "k": 20, "fixed_reads": 6_001}, 0),
    "pe_fixed_reads_candidates": (sim.SimConfig(seed=124, genome_length=50_000, num_reads=10_000, paired=True,
                                                repeat_families=3, repeat_copies=3),
                                  {"coverage": 30, "k": 20, "paired": True, "candidates": True,
                                   "fixed_reads": 4_000}, 0),
}


def md5(b: bytes) -> str:
    return hashlib.md5(b).hexdigest()


def fastq_sequences(path: str, n: int) -> list[bytes]:
    with open(path, "rb") as f:
        lines = f.read().split(b"\n")
    seqs = lines[1::4]
    assert len(seqs) >= n, (path, len(seqs), n)
    return seqs[:n]


def run_case(name: str, cfg: sim.SimConfig, opts: dict, stage_anchors: int, work: str, threads: int) -> dict:
    reads = sim.SimReads(cfg)
    d = os.path.join(work, name)
    os.makedirs(d, exist_ok=True)
    paired = opts.get("paired", False)
    if paired:
        in1, in2 = os.path.join(d, "in_1.fq"), os.path.join(d, "in_2.fq")
        reads.write_fastq(in1, in2)
        inputs = [in1, in2]
    else:
        in1 = os.path.join(d, "in.fq")
        reads.write_fastq(in1)
        inputs = [in1]
    cmd = [os.path.join(REPO, "oracle", "_ref", "ref_care"), "-d", d, "-c", str(opts["coverage"]),
           "-k", str(opts["k"]), "-h", str(opts.get("maps", 48)), "-t", str(threads)]
    for i, p in enumerate(inputs):
        cmd += ["-i", p, "-o", f"out_{i}.fq"]
    if opts.get("quality"):
        cmd.append("-q")
    if opts.get("exclude_ambiguous"):
        cmd.append("--exclude-ambiguous")
    if paired:
        cmd.append("--pe")
    if opts.get("candidates"):
        cmd.append("--candidates")
    if "new_columns" in opts:
        cmd += ["--new-columns", str(opts["new_columns"])]
    if "quality_bits" in opts:
        cmd += ["--quality-bits", str(opts["quality_bits"])]
    if "fixed_reads" in opts:
        cmd += ["--fixed-reads", str(opts["fixed_reads"])]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed on {name}:\n{r.stdout[-3000:]}")
    # the same run with " care:q=N" header labels, into its own directory
    ld = os.path.join(d, "labels")
    os.makedirs(ld, exist_ok=True)
    lcmd = list(cmd)
    lcmd[lcmd.index("-d") + 1] = ld
    r = subprocess.run(lcmd + ["--labels"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference (labels) failed on {name}:\n{r.stdout[-3000:]}")
    labels_md5 = []
    for i in range(len(inputs)):
        with open(os.path.join(ld, f"out_{i}.fq"), "rb") as f:
            labels_md5.append(md5(f.read()))
    # output sequences in read-id order (paired: interleave file 1 and file 2)
    if paired:
        s1 = fastq_sequences(os.path.join(d, "out_0.fq"), reads.n // 2)
        s2 = fastq_sequences(os.path.join(d, "out_1.fq"), reads.n // 2)
        outs = [x for pair in zip(s1, s2) for x in pair]
    else:
        outs = fastq_sequences(os.path.join(d, "out_0.fq"), reads.n)
    out_all = np.frombuffer(b"".join(outs), dtype=np.uint8)
    assert out_all.shape == reads.sequences.shape
    # edits: every position where the reference's output differs from the input,
    # as (read id, position in read, output base)
    diff = np.nonzero(out_all != reads.sequences)[0]
    rid = (np.searchsorted(reads.offsets, diff, side="right") - 1).astype(np.uint32)
    pos = (diff - reads.offsets[rid]).astype(np.uint16)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), read=np.diff(rid, prepend=np.uint32(0)).astype(np.uint32),
                        pos=pos, base=out_all[diff])
    changed = np.unique(rid)
    out_files = [os.path.join(d, f"out_{i}.fq") for i in range(len(inputs))]
    in_files_md5 = []
    for pth in inputs:
        with open(pth, "rb") as f:
            in_files_md5.append(md5(f.read()))
    out_files_md5 = []
    for pth in out_files:
        with open(pth, "rb") as f:
            out_files_md5.append(md5(f.read()))
    entry = {
        "config": dataclasses.asdict(cfg),
        "options": opts,
        "num_reads": reads.n,
        "input_file_md5": in_files_md5,
        "output_file_md5": out_files_md5,
        "labels_file_md5": labels_md5,
        "input_md5": md5(reads.sequences.tobytes()),
        "input_qual_md5": md5(reads.qualities.tobytes()),
        "output_md5": md5(out_all.tobytes()),
        "changed_reads": int(len(changed)),
        "score": reads.score(out_all),
    }
    if stage_anchors:
        st = os.path.join(d, "stages.txt")
        scmd = [os.path.join(REPO, "oracle", "_ref", "ref_stages"), "-i", in1, "-c", str(opts["coverage"]),
                "-k", str(opts["k"]), "--first", "0", "--last", str(stage_anchors), "--sigreads", "40",
                "--out", st]
        if opts.get("quality"):
            scmd.append("-q")
        r = subprocess.run(scmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"stage dump failed on {name}:\n{r.stdout[-3000:]}")
        with open(st, "rb") as f, gzip.GzipFile(os.path.join(HERE, f"{name}.stages.txt.gz"), "wb", compresslevel=9,
                                                mtime=0) as g:
            shutil.copyfileobj(f, g)
        entry["stage_anchors"] = stage_anchors
    return entry


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    import oracle
    if not oracle.build_reference(args.ref):
        sys.exit(f"reference tree not found at {args.ref or oracle.reference_dir()}")
    manifest_path = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(manifest_path)) if os.path.exists(manifest_path) else {}
    with tempfile.TemporaryDirectory() as work:
        for name, (cfg, opts, stages) in CASES.items():
            if args.only and name not in args.only:
                continue
            manifest[name] = run_case(name, cfg, opts, stages, work, args.threads)
            print(name, manifest[name]["changed_reads"], manifest[name]["score"], flush=True)
    with open(manifest_path, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
