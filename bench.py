"""Benchmark of the CARE correction hot path on one GB300 (or N replicas).

Workload (default): the 10 Mbp genome with 200 diverged repeat copies, 2M x
150 bp single-end reads at 30x, substitution rate rising 0.2% -> 2% from 5'
to 3' (seeded synthetic data of that shape; k=20, 48 maps, coverage 30).

One step = correction of every anchor of that read set.  Four forms are
timed, each on its own context with the same reads:
  plain            stage kernels per batch, classic decision (bit-exact with the
                   reference)
  batched          captured per-batch graphs with persistent work-stealing
                   kernels, classic decision (bit-exact with plain)
  batched_learned  the batched driver with the learned decision (the trained
                   classifier shipped with the package)
  batched_candidates  the batched driver with candidate correction
                   (--candidateCorrection; the combine step follows cg_correct)
and for each the base-level TP/FP/FN against the generator's truth (also for
the forest decision, untimed).
  value  corrected reads/s of batched_learned with the read store and hash
         tables resident in HBM (device time of cg_correct, CUDA events on the
         library's streams); forms[...] has the same for every form
  e2e    the same metric through the public C ABI with host buffers: append the
         reads from host memory, build the store and the tables on the device,
         load the classifier, correct every anchor and copy every result back
         to host memory
The read store (0.5 GB) and tables (several GB) exceed the 129 MB L2, so no
separate flush is needed between steps.

`--impl reference` times the reference algorithm on the host cores: the
reference's own build does not exist on the GPU machine, so this arm runs the
CPU restatement of it (oracle/, bit-exact with the reference on the committed
fixtures) with all host threads, each step a bounded sample of anchors.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from rabbitqcplus_gb300 import capi, learned, sim  # noqa: E402

METRIC = "corrected reads/s on 1 GB300: plain vs batched+learned, at equal TP/FP vs truth"
# DRAM bytes (read + write) of align_lane_kernel per candidate, measured by ncu on one
# 65536-anchor launch of this workload at 2 Mbp: 91.59 MB for 3.777M candidates
ALIGN_DRAM_BYTES_PER_CANDIDATE = 91.59e6 / 3.777e6
UNIT = "reads/s"


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int, paused: bool = False):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._active = threading.Event()
        if not paused:
            self._active.set()
        self._t = None

    def pause(self):
        self._active.clear()

    def resume(self):
        self._active.set()

    def _run(self):
        while not self._stop.is_set():
            if not self._active.is_set():
                self._stop.wait(0.05)
                continue
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.samples.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and
                          s[3 + i].lower() in ("active", "1")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_arm(reads, opts, sample_anchors: int, threads: int, seconds_target: float = 15.0):
    """Reference algorithm (oracle restatement) on host cores over a bounded anchor sample."""
    import oracle
    t0 = time.perf_counter()
    orc = oracle.Oracle(opts, reads.sequences, reads.offsets, None, threads=threads)
    build_s = time.perf_counter() - t0
    # grow the sample until it takes a few seconds, capped by seconds_target
    n = min(sample_anchors, reads.n)
    first = reads.n // 3
    t0 = time.perf_counter()
    probe = min(2000, n, reads.n - first)
    orc.correct(first, probe, threads=threads)
    dt = time.perf_counter() - t0
    rate = probe / max(dt, 1e-6)
    n = int(min(n, max(2000, rate * seconds_target), reads.n - first))
    t0 = time.perf_counter()
    orc.correct(first, n, threads=threads)
    dt = time.perf_counter() - t0
    orc.close()
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} anchors (ids {first}..{first + n - 1}) of the workload against its full "
                      f"hash tables; table build {build_s:.1f}s not included"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c1_10mbp_repeats_se")
    ap.add_argument("--genome", type=int, default=0, help="scale the config to this genome length")
    ap.add_argument("--cpu-sample", type=int, default=200_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    rank, world, local = env_rank()
    threads = os.cpu_count() or 1

    cfg = sim.scaled(args.config, args.genome) if args.genome else sim.CONFIGS[args.config]
    coverage = round(cfg.num_reads * (cfg.read_len_min + cfg.read_len_max) / 2 / cfg.genome_length)
    opts = capi.CareOptions.defaults(float(coverage), kmerlength=20,
                                     pair_mode=capi.CG_PAIR_PE if cfg.paired else capi.CG_PAIR_SE)
    config = {"workload": f"{args.config}: genome {cfg.genome_length} bp, {cfg.num_reads} reads "
                          f"{cfg.read_len_min}-{cfg.read_len_max} bp, {coverage}x, k=20, 48 maps",
              "reads": cfg.num_reads, "coverage": coverage, "kmerlength": 20, "hashmaps": 48,
              "paired": bool(cfg.paired), "l2": "inputs larger than L2 (read store + tables > 129 MB)"}

    if args.impl == "reference":
        if rank != 0:
            return
        reads = sim.SimReads(cfg)
        vals = []
        for i in range(args.warmup + args.steps):
            r = cpu_arm(reads, capi.CareOptions.defaults(float(coverage), kmerlength=20), args.cpu_sample,
                        threads, seconds_target=8.0)
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": r["sample"]},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    reads = sim.SimReads(cfg)
    opts.device = local

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    model = open(learned.DEFAULT_MODEL, "rb").read()
    forest = open(os.path.join(REPO, "tests", "golden", "forest_anchor.bin"), "rb").read()
    n_total = reads.n

    def form_options(form):
        o = capi.CareOptions.defaults(opts.estimated_coverage, kmerlength=20, pair_mode=opts.pair_mode,
                                      device=local)
        if form in ("batched", "batched_learned", "batched_candidates"):
            o.driver = capi.CG_DRIVER_BATCHED
        if form == "batched_candidates":
            o.correct_candidates = 1
        if form == "batched_learned":
            o.correction_type = capi.CG_CORR_LEARNED
        if form == "forest":
            o.correction_type = capi.CG_CORR_FOREST
        return o

    def make_ctx(form):
        g = capi.CareGpu(form_options(form))
        g.append_reads(reads.sequences, reads.offsets)
        g.build_tables()
        if form == "batched_learned":
            g.load_classifier(model)
        if form == "forest":
            g.load_forest(forest)
        return g

    flags = np.zeros(n_total, np.uint8)
    out = None

    def run_form(form, steps, warmup, clk=None):
        """Resident correction: build once, then time `steps` full passes (device time of cg_correct)."""
        nonlocal out
        g = make_ctx(form)
        n, lmax = g.read_info()
        if out is None:
            out = np.zeros((n, lmax), np.uint8)
        for _ in range(warmup):
            g.correct(0, n, flags, out)
        st0 = g.stats()
        barrier()
        if clk:
            clk.resume()
        t0 = time.perf_counter()
        dev = 0.0
        for _ in range(steps):
            g.correct(0, n, flags, out)
            dev += g.stats()["seconds_correct"]
        barrier()
        wall = time.perf_counter() - t0
        if clk:
            clk.pause()
        st1 = g.stats()
        final = capi.apply_corrections(reads.sequences, reads.offsets, flags, out)
        g.close()
        t = torch.tensor([dev], dtype=torch.float64, device="cuda")
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev = float(t.item())
        return {"n": n, "lmax": lmax, "dev": dev, "wall": wall, "st0": st0, "st1": st1, "score": reads.score(final),
                "flags": flags.copy() if form in ("plain", "batched") else None,
                "out": out.copy() if form in ("plain", "batched") else None}

    hbm_peak, peak_kind = measured_peaks()

    def alg_bytes(r, steps):
        # algorithmic bytes of one pass (per anchor: its 2-bit row 40 B, 48 keys 384 B, 48 lookup slots
        # 768 B, 4 B per raw id, 44 B per unique candidate (row + length), the output record)
        d = {k: (r["st1"][k] - r["st0"][k]) / steps for k in ("raw_candidate_ids", "unique_candidates")}
        pitch = (r["lmax"] + 15) // 16
        return r["n"] * (4 * pitch + 48 * 8 + 48 * 16 + r["lmax"] + 1) + 4 * d["raw_candidate_ids"] + \
            (4 * pitch + 4) * d["unique_candidates"]

    def summary(r, steps):
        sec = r["dev"] / steps
        b = alg_bytes(r, steps)
        return {"value": world * r["n"] / sec, "unit": UNIT, "ms_per_step": sec * 1e3,
                "alg_gbs": b / sec / 1e9, "hbm_frac": b / sec / 1e9 / hbm_peak,
                "tp": r["score"]["tp"], "fp": r["score"]["fp"], "fn": r["score"]["fn"],
                "gpu_launches_per_step": (r["st1"]["kernel_launches"] - r["st0"]["kernel_launches"]) / steps}

    clk = ClockSampler(local, paused=True)
    with clk:
        plain = run_form("plain", args.steps, args.warmup, clk)
        bat = run_form("batched", args.steps, args.warmup, clk)
        bl = run_form("batched_learned", args.steps, args.warmup, clk)
        cand = run_form("batched_candidates", args.steps, args.warmup, clk)
    forest_run = run_form("forest", 1, 0)
    st0, st1 = bl["st0"], bl["st1"]
    n = bl["n"]
    lmax = bl["lmax"]
    dev_seconds = bl["dev"]
    value = world * n * args.steps / dev_seconds
    launches = st1["kernel_launches"] - st0["kernel_launches"]
    same = bool(np.array_equal(plain["flags"], bat["flags"]))
    if same:
        idx = np.nonzero(plain["flags"] & capi.CG_RESULT_CORRECTED)[0]
        lens = reads.lengths[idx]
        po, bo = plain["out"][idx], bat["out"][idx]
        mask = np.arange(lmax)[None, :] < lens[:, None]
        same = bool(np.array_equal(np.where(mask, po, 0), np.where(mask, bo, 0)))
    forms = {"plain": summary(plain, args.steps), "batched": summary(bat, args.steps),
             "batched_learned": summary(bl, args.steps),
             # --candidateCorrection: device time of cg_correct; the combine step after it is one
             # thread per read
             "batched_candidates": summary(cand, args.steps),
             "forest": {"tp": forest_run["score"]["tp"], "fp": forest_run["score"]["fp"],
                        "fn": forest_run["score"]["fn"], "driver": "plain", "timed": False},
             "batched_bit_exact_with_plain": same,
             "batched_shape": {k: bl["st1"][k] for k in ("batch_anchors", "align_blocks", "msa_warps", "streams",
                                                       "seconds_tune")}}

    # roofline of the dominant kernel, from the plain form's per-stage CUDA events (the
    # batched form runs the same kernels inside graph replays, where they are not timed apart)
    p0, p1 = plain["st0"], plain["st1"]
    stages = {"align": p1["seconds_align"] - p0["seconds_align"],
              "filter": p1["seconds_filter"] - p0["seconds_filter"],
              "msa": p1["seconds_msa"] - p0["seconds_msa"],
              "candidates": p1["seconds_candidates"] - p0["seconds_candidates"]}
    dom = max(stages, key=stages.get)
    per_step_cands = (p1["unique_candidates"] - p0["unique_candidates"]) / args.steps
    per_step_msa = (p1["msa_candidates"] - p0["msa_candidates"]) / args.steps
    wp = (lmax + 31) // 32 + 1
    pitch = (lmax + 15) // 16
    if dom == "align":
        # align_lane_kernel, per candidate: its id (4 B) and length (2 B), its forward and
        # reverse-complement hi/lo planes (4*wp words), the packed result (8 B);
        # per anchor: its forward planes (2*wp words), length and two offsets (10 B)
        bytes_step = per_step_cands * (4 + 2 + 16 * wp + 8) + n * (8 * wp + 10)
        launches_k = (p1["align_launches"] - p0["align_launches"])
        kname = "align_lane_kernel"
    elif dom == "msa":
        # msa_warp_kernel, per kept candidate: its record (id, shift, length, orientation,
        # weight = 13 B) and its 2-bit row; per anchor: its 2-bit row, length, the
        # corrected bases and flags written
        bytes_step = per_step_msa * (13 + 4 * pitch) + n * (4 * pitch + 2 + lmax + 1)
        launches_k = (p1["msa_launches"] - p0["msa_launches"])
        kname = "msa_warp_kernel"
    else:
        bytes_step = (p1["raw_candidate_ids"] - p0["raw_candidate_ids"]) / args.steps * 4 + n * 48 * 24
        launches_k = max(p1["align_launches"] - p0["align_launches"], 1)
        kname = "gather_unique_kernel"
    dur = stages[dom] / max(launches_k, 1)
    kernel_bytes_launch = bytes_step * args.steps / max(launches_k, 1)
    # The path's algorithmic bytes per anchor (the scope's per-unit figure):
    # 2-bit anchor row, 48 signature keys and 48 lookup slots probed, the raw
    # ids (4 B each) and the unique candidates' rows and lengths (44 B each,
    # at 150 bp), and the result written (flag and corrected bases); one
    # launch of the dominant kernel processes the anchors of one batch.
    per_step_raw = (p1["raw_candidate_ids"] - p0["raw_candidate_ids"]) / args.steps
    path_bytes_step = n * (4 * pitch + 48 * 8 + 48 * 16 + 1 + lmax) + 4 * per_step_raw + \
        per_step_cands * (4 * pitch + 4)
    bytes_launch = path_bytes_step * args.steps / max(launches_k, 1)
    achieved = bytes_launch / dur / 1e9
    traffic = None
    if dom == "align":
        # DRAM bytes per candidate measured by ncu (ALIGN_DRAM_BYTES_PER_CANDIDATE), scaled by the
        # candidates of an average launch (the traffic grows with the candidates processed)
        traffic = ALIGN_DRAM_BYTES_PER_CANDIDATE * per_step_cands * args.steps / max(launches_k, 1)
    roof = {"bound": "hbm", "kernel": kname, "form": "plain", "achieved": achieved, "peak": hbm_peak,
            "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": bytes_launch,
            "algorithmic_bytes_per_anchor": path_bytes_step / max(n, 1),
            "kernel_bytes_per_launch": kernel_bytes_launch,
            "avg_launch_ms": dur * 1e3,
            "stage_seconds_per_step": {k: v / args.steps for k, v in stages.items()},
            "note": "integer-pipe bound (ALU pipe 75% active in ncu); the fraction is of the HBM roofline, and "
                    "traffic (measured DRAM bytes) is below the algorithmic bytes because candidate planes "
                    "shared between anchors hit in L2"}

    # e2e through the C ABI with host buffers (batched + learned)
    e2e = None
    if not args.no_e2e:
        # one untimed step, then `steps` timed ones, each through a fresh context
        for i in range(1 + args.steps):
            barrier()
            if i == 1:
                t0 = time.perf_counter()
            g2 = make_ctx("batched_learned")
            g2.correct(0, n, flags, out)
            g2.close()
        barrier()
        te = time.perf_counter() - t0
        tt = torch.tensor([te], dtype=torch.float64, device="cuda")
        if dist is not None:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e = {"value": world * n * args.steps / float(tt.item()), "unit": UNIT, "steps": args.steps,
               "h2d_bytes_per_step": int(reads.sequences.nbytes + reads.offsets.nbytes + len(model)),
               "d2h_bytes_per_step": int(flags.nbytes + out.nbytes),
               "form": "batched_learned",
               "includes": "append from host, device read-store + table build, classifier load, correction, "
                           "results to host (launch shapes tuned in the warm-up)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_arm(reads, capi.CareOptions.defaults(float(coverage), kmerlength=20), args.cpu_sample, threads)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_seconds / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": config, "form": "batched_learned", "forms": forms, "e2e": e2e,
                "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                "wall_seconds_timed": bl["wall"], "build_seconds": st1["seconds_build"],
                "score": bl["score"], "stats": {k: st1[k] for k in ("raw_candidate_ids", "unique_candidates",
                                                                    "aligned_candidates", "msa_candidates",
                                                                    "msa_builds", "corrected_anchors", "hq_anchors", "table_keys",
                                                                    "table_values", "learned_columns",
                                                                    "learned_corrections")}}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
