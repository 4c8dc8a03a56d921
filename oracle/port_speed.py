"""ORACLE -- test infrastructure, not product code.

Speed of the CPU restatement (oracle/care_oracle.cpp, the "port") against the
reference's own build (oracle/_ref/ref_care, compiled from the reference's
sources by oracle/ref.mk) on the same generated workload and thread count:
STEP2 (the correction of every anchor) only, tables built beforehand by each.

    python oracle/port_speed.py [--config c1_10mbp_repeats_se] [--threads 8]

The reference's STEP2 figure is its own "Correction throughput" print
(src/dispatch_care_correct_cpu.cpp:159-169: reads / the STEP2 timer, which
includes up to 1 s of its progress thread's sleep); the port's is the wall
time of Oracle.correct over every anchor.  Both outputs are compared byte for
byte.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from rabbitqcplus_gb300 import capi, sim  # noqa: E402


def compare(config: str, threads: int) -> dict:
    """Both implementations on one generated workload: STEP2 speeds and
    whether the corrected outputs are byte-identical."""
    exe = os.path.join(HERE, "_ref", "ref_care")
    if not os.path.exists(exe) and not oracle.build_reference():
        raise RuntimeError("the reference build (oracle/_ref/ref_care) is not available")
    cfg = sim.CONFIGS[config]
    reads = sim.SimReads(cfg)
    cov = round(cfg.num_reads * (cfg.read_len_min + cfg.read_len_max) / 2 / cfg.genome_length)
    with tempfile.TemporaryDirectory() as d:
        fq = os.path.join(d, "in.fq")
        reads.write_fastq(fq)
        r = subprocess.run([exe, "-i", fq, "-o", "out.fq", "-d", d, "-c", str(cov), "-k", "20",
                            "-t", str(threads)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout[-3000:])
        m = re.search(r"Correction throughput : ~([0-9.eE+]+) reads/second", r.stdout)
        ref_rate = float(m.group(1))
        with open(os.path.join(d, "out.fq"), "rb") as f:
            ref_seqs = f.read().split(b"\n")[1::4][:reads.n]
    opts = capi.CareOptions.defaults(float(cov), kmerlength=20)
    orc = oracle.Oracle(opts, reads.sequences, reads.offsets, None, threads=threads)
    t0 = time.perf_counter()
    flags, seqs, _ = orc.correct()
    port_s = time.perf_counter() - t0
    out = capi.apply_corrections(reads.sequences, reads.offsets, flags, seqs)
    same = out.tobytes() == b"".join(ref_seqs)
    cpu = platform.processor() or platform.machine()
    try:
        with open("/proc/cpuinfo") as f:
            names = [ln.split(":", 1)[1].strip() for ln in f if ln.startswith("model name")]
        cpu = names[0] if names else cpu
    except OSError:
        pass
    return {"config": config, "reads": reads.n, "threads": threads, "cpu": cpu,
            "reference_step2_reads_per_s": ref_rate, "port_step2_reads_per_s": reads.n / port_s,
            "port_over_reference": reads.n / port_s / ref_rate, "outputs_identical": bool(same)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1_10mbp_repeats_se")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    print(json.dumps(compare(args.config, args.threads)))


if __name__ == "__main__":
    main()
