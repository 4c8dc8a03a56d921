"""Benchmark of the CARE correction hot path on one GB300 (or N replicas).

Workload (default, `--config c4_500mbp_se`): a 500 Mbp genome with 5% repeat
content, 100M x 150 bp single-end reads at 30x, 1% substitutions, Phred
qualities as the other workloads (seeded synthetic data of that shape: no
public dataset is available offline); k = 20, 48 maps, coverage 30.  The read
store, the 48 hash tables and the signatures of all 100M reads stay resident in
HBM (inputs far larger than the 129 MB L2, so no flush is needed between
steps).

One step = the correction of one window of anchors (4,194,304 by default)
against the tables of the whole read set; the steps walk through the read
set window by window (warm-up steps first), so `--warmup 5 --steps 20` covers
every anchor once.  Forms, each on its own context with the same reads:
  plain               stage kernels per batch, classic decision (bit-exact
                      with the reference)
  batched             captured per-batch graphs with persistent
                      work-stealing kernels, classic decision (bit-exact with
                      plain)
  batched_learned     the batched driver with the learned decision (the
                      trained classifier shipped with the package) -- `value`
  batched_candidates  the batched driver with candidate correction
                      (--candidateCorrection)
TP/FP/FN (bases, against the generator's truth) come from an untimed full
pass of each form over every read (with the combine step for candidate
correction), and from the forest decision (plain driver, untimed).

  value   corrected reads/s of batched_learned over the timed windows (device
          time of cg_correct, CUDA events on the library's streams, data
          resident in HBM); forms[...] has the same for every form
  e2e     the same metric end to end through the public C ABI from pinned
          host buffers: per step a fresh context appends every read, builds
          the read store and the tables on the device, loads the classifier,
          corrects every anchor and copies every result back to pinned host
          memory
  roofline the dominant kernel of the plain form (CUDA events per stage) in
          HBM bytes, plus its integer-issue fraction
  cpu_baseline  the reference algorithm (oracle/, bit-exact restatement of
          the reference's CPU path, pinned to its output) on every host core,
          over a bounded sample of anchors of the same workload (tables built
          once, not timed)
  secondary  the same forms and e2e on the 2M-read, 10 Mbp workload with repeats

`--impl reference` times the reference algorithm on the host cores: the
reference's own build does not exist on the GPU machine, so this arm runs the
CPU restatement of it (oracle/, bit-exact with the reference; its speed
against the reference's own build, measured where both exist, is
PORT_VS_REFERENCE below) with all host threads: tables built once per
process, then each step a fixed slice of anchors.
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

from rabbitqcplus_gb300 import capi, learned, shard, sim  # noqa: E402

METRIC = "corrected reads/s on 1 GB300: plain vs batched+learned, at equal TP/FP vs truth"
UNIT = "reads/s"
WINDOW = 4_194_304  # anchors per step
# DRAM bytes (read + write) of align_lane_kernel per candidate, its warp
# instructions per candidate and its ALU pipe activity, measured by ncu on one
# 65536-anchor launch of the 100M-read workload's shape at 20 Mbp
# (profiles/align_lane_kernel_c4_shape_20mbp.md: 738.1 MB and 7.67810e8 warp
# instructions for the launch's 3.3555M candidates, ALU pipe 84.9% active).
# On the 2M-read workload with repeats the DRAM bytes per candidate are far
# fewer (candidates shared by the anchors of a batch hit in L2 there).
ALIGN_DRAM_BYTES_PER_CANDIDATE = 738.1e6 / 3.3555e6
ALIGN_WARP_INST_PER_CANDIDATE = 7.67810e8 / 3.3555e6
ALIGN_ALU_PIPE_ACTIVE = 0.849
# STEP2 speed of the oracle (the port) over the reference's own build, both on
# 8 threads of an Intel Xeon @ 2.70 GHz, 2M-read 150 bp workload with repeats,
# outputs byte-identical (python oracle/port_speed.py --threads 8): the port
# corrects 18.9k reads/s where the reference corrects 21.3k, so a GPU/port
# ratio overstates the GPU/reference ratio by about 1.12x
PORT_VS_REFERENCE = {"port_over_reference": 0.889, "port_reads_per_s": 18911, "reference_reads_per_s": 21274,
                     "threads": 8, "workload": "c1_10mbp_repeats_se (2M reads)",
                     "how": "python oracle/port_speed.py --threads 8, reference built from its sources by oracle/ref.mk"}


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


def coverage_of(cfg: sim.SimConfig) -> int:
    return round(cfg.num_reads * (cfg.read_len_min + cfg.read_len_max) / 2 / cfg.genome_length)


def windows_of(n: int, w: int, paired: bool):
    w = max(2, w & ~1) if paired else max(1, w)
    return [(s, min(w, n - s)) for s in range(0, n, w)]


def workload_desc(name: str, cfg: sim.SimConfig) -> dict:
    cov = coverage_of(cfg)
    return {"workload": f"{name}: genome {cfg.genome_length} bp, {cfg.num_reads} reads "
                        f"{cfg.read_len_min}-{cfg.read_len_max} bp{' paired' if cfg.paired else ''}, {cov}x, "
                        f"k=20, 48 maps",
            "reads": cfg.num_reads, "coverage": cov, "kmerlength": 20, "hashmaps": 48, "paired": bool(cfg.paired),
            "l2": "inputs larger than L2 (read store + tables > 129 MB); no flush"}


class Oracle1:
    """The oracle's tables of one read set, built once; slices of anchors timed."""

    def __init__(self, reads, cfg, threads):
        import oracle
        self.threads = threads
        opts = capi.CareOptions.defaults(float(coverage_of(cfg)), kmerlength=20,
                                         pair_mode=capi.CG_PAIR_PE if cfg.paired else capi.CG_PAIR_SE)
        t0 = time.perf_counter()
        self.orc = oracle.Oracle(opts, reads.sequences, reads.offsets, None, threads=threads)
        self.build_s = time.perf_counter() - t0
        self.n = reads.n
        self.paired = bool(cfg.paired)

    def slice_size(self, seconds: float) -> int:
        """Anchors that take about `seconds` on the host cores (probed)."""
        first = (self.n // 3) & ~1
        probe = min(20_000, self.n - first) & ~1
        t0 = time.perf_counter()
        self.orc.correct(first, probe, threads=self.threads)
        rate = probe / max(time.perf_counter() - t0, 1e-6)
        return max(2000, min(int(rate * seconds), self.n // 2)) & ~1

    def time_slice(self, first: int, count: int) -> float:
        first = min(first, self.n - count) & ~1
        t0 = time.perf_counter()
        self.orc.correct(first, count, threads=self.threads)
        return time.perf_counter() - t0

    def close(self):
        self.orc.close()


def cpu_baseline(reads, cfg, threads, seconds=15.0):
    o = Oracle1(reads, cfg, threads)
    count = o.slice_size(seconds / 3)
    first = (reads.n // 3) & ~1
    dt = o.time_slice(first, count * 3)
    o.close()
    return {"value": count * 3 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{count * 3} anchors (ids {first}..{first + count * 3 - 1}) of the workload against the "
                      f"tables of all {reads.n} reads (built once in {o.build_s:.1f} s, not timed)",
            "port_vs_reference_step2": PORT_VS_REFERENCE}


def reference_arm(args, cfg, name, threads):
    reads = sim.SimReads(cfg)
    o = Oracle1(reads, cfg, threads)
    count = o.slice_size(4.0)
    total_anchors, total_s = 0, 0.0
    for i in range(args.warmup + args.steps):
        first = (i * count * 7919) % max(reads.n - count, 1)  # slices spread over the read set
        dt = o.time_slice(first, count)
        if i >= args.warmup:
            total_anchors += count
            total_s += dt
    o.close()
    v = total_anchors / total_s
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_desc(name, cfg), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step {count} anchors of the workload against the tables of all "
                                       f"{reads.n} reads (built once in {o.build_s:.1f} s, not timed)",
                             "port_vs_reference_step2": PORT_VS_REFERENCE},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c4_500mbp_se")
    ap.add_argument("--genome", type=int, default=0, help="scale the config to this genome length")
    ap.add_argument("--window", type=int, default=WINDOW, help="anchors per step")
    ap.add_argument("--secondary", default="c1_10mbp_repeats_se", help="second workload ('none' to skip)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--forms", default="plain,batched,batched_learned,batched_candidates")
    ap.add_argument("--sweep", default="c1_10mbp_repeats_se,c3_10mbp_varlen",
                    help="workloads of the forest/learned threshold sweep ('none' to skip)")
    args = ap.parse_args()
    rank, world, local = env_rank()
    threads = os.cpu_count() or 1
    cfg = sim.scaled(args.config, args.genome) if args.genome else sim.CONFIGS[args.config]

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, cfg, args.config, threads)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    model = open(learned.DEFAULT_MODEL, "rb").read()
    # the forest the learned decision is compared with: trained on the reference's
    # Print-mode features of the learned classifier's own training reads
    # (tests/golden/make_forest.py workload); the fixture forest if it is absent
    forest_path = os.path.join(REPO, "tests", "golden", "forest_varlen.bin")
    if not os.path.exists(forest_path):
        forest_path = os.path.join(REPO, "tests", "golden", "forest_anchor.bin")
    forest = open(forest_path, "rb").read()
    hbm_peak, peak_kind = measured_peaks()
    forms_wanted = [f for f in args.forms.split(",") if f]
    if "batched_learned" not in forms_wanted:
        forms_wanted.append("batched_learned")

    def form_options(cfg_, form):
        o = capi.CareOptions.defaults(float(coverage_of(cfg_)), kmerlength=20, device=local,
                                      pair_mode=capi.CG_PAIR_PE if cfg_.paired else capi.CG_PAIR_SE)
        if form in ("batched", "batched_learned", "batched_candidates"):
            o.driver = capi.CG_DRIVER_BATCHED
        if form == "batched_candidates":
            o.correct_candidates = 1
        if form == "batched_learned":
            o.correction_type = capi.CG_CORR_LEARNED
        if form == "forest":
            o.correction_type = capi.CG_CORR_FOREST
        return o

    def make_ctx(reads, cfg_, form, seqs=None, offs=None):
        g = capi.CareGpu(form_options(cfg_, form))
        g.append_reads(reads.sequences if seqs is None else seqs, reads.offsets if offs is None else offs)
        g.build_tables()
        if form == "batched_learned":
            g.load_classifier(model)
        if form == "forest":
            g.load_forest(forest)
        return g

    def window_digest(flags, rows, lengths):
        """Order-dependent checksum of a window's flags and corrected bases (rows
        of uncorrected anchors and bytes past a read's end do not count)."""
        L = rows.shape[1]
        w = (np.arange(1, L + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)) | np.uint64(1)
        corr = (flags & capi.CG_RESULT_CORRECTED) != 0
        h = int(np.sum(flags.astype(np.uint64) * np.arange(1, flags.size + 1, dtype=np.uint64)))
        idx = np.nonzero(corr)[0]
        for a in range(0, idx.size, 1 << 18):
            sl = idx[a:a + (1 << 18)]
            m = np.arange(L)[None, :] < lengths[sl][:, None]
            v = np.where(m, rows[sl], 0).astype(np.uint64)
            h = (h * 1000003 + int(np.sum((v * w[None, :]).sum(axis=1) * (sl.astype(np.uint64) + np.uint64(1))))) \
                & 0xFFFFFFFFFFFFFFFF
        return h

    def score_pass(g, reads, wins, lmax, digest=False):
        """Untimed pass over every window; TP/FP/FN of the whole read set (and
        per-window checksums of the results)."""
        cand = bool(g.options.correct_candidates)
        if cand:
            # the combine step needs the pass over every read: every rank scores the whole set
            wins = windows_of(reads.n, args.window, bool(reads.cfg.paired))
        wmax = max(c for _, c in wins)
        if cand:
            flags_all = np.zeros(reads.n, np.uint8)
            rows_all = np.zeros((reads.n, lmax), np.uint8)
            for s, c in wins:
                g.correct(s, c, flags_all[s:s + c], rows_all[s:s + c], combine=False)
            g.combine(0, flags_all)
            return reads.score_results(0, flags_all, rows_all), None
        flags = np.zeros(wmax, np.uint8)
        rows = np.zeros((wmax, lmax), np.uint8)
        tot = {"tp": 0, "fp": 0, "fn": 0, "reads_scored": 0}
        digests = []
        for s, c in wins:
            g.correct(s, c, flags[:c], rows[:c])
            sc = reads.score_results(s, flags[:c], rows[:c])
            for k in tot:
                tot[k] += sc[k]
            if digest:
                digests.append(window_digest(flags[:c], rows[:c], reads.lengths[s:s + c]))
        if dist is not None:  # the ranks' shards together cover every read
            t = torch.tensor([tot[k] for k in ("tp", "fp", "fn", "reads_scored")], dtype=torch.int64, device="cuda")
            dist.all_reduce(t)
            tot = dict(zip(("tp", "fp", "fn", "reads_scored"), (int(x) for x in t.tolist())))
        return tot, (digests if digest else None)

    def run_form(reads, cfg_, form, wins, steps, warmup, clk=None, digest=False):
        g = make_ctx(reads, cfg_, form)
        n, lmax = g.read_info()
        wmax = max(c for _, c in wins)
        flags = np.zeros(wmax, np.uint8)
        rows = np.zeros((wmax, lmax), np.uint8)
        dev, anchors = 0.0, 0
        st0 = None
        wall0 = 0.0
        for i in range(warmup + steps):
            if i == warmup:
                barrier()
                if clk:
                    clk.resume()
                st0 = g.stats()
                wall0 = time.perf_counter()
            s, c = wins[i % len(wins)]
            g.correct(s, c, flags[:c], rows[:c], combine=False)
            if i >= warmup:
                dev += g.stats()["seconds_correct"]
                anchors += c
        barrier()
        wall = time.perf_counter() - wall0
        if clk:
            clk.pause()
        st1 = g.stats()
        sc, res = score_pass(g, reads, wins, lmax, digest)
        g.close()
        return {"n": n, "lmax": lmax, "dev": max_over_ranks(dev), "anchors": anchors, "wall": wall, "st0": st0,
                "st1": st1, "score": sc, "res": res}

    def summary(r):
        sec = r["dev"]
        d = {k: (r["st1"][k] - r["st0"][k]) for k in ("raw_candidate_ids", "unique_candidates", "kernel_launches")}
        pitch = (r["lmax"] + 15) // 16
        b = r["anchors"] * (4 * pitch + 48 * 8 + 48 * 16 + r["lmax"] + 1) + 4 * d["raw_candidate_ids"] + \
            (4 * pitch + 4) * d["unique_candidates"]
        return {"value": world * r["anchors"] / sec, "unit": UNIT, "ms_per_step": sec / max(r["steps"], 1) * 1e3,
                "alg_gbs": b / sec / 1e9, "hbm_frac": b / sec / 1e9 / hbm_peak,
                "tp": r["score"]["tp"], "fp": r["score"]["fp"], "fn": r["score"]["fn"],
                "gpu_launches_per_step": d["kernel_launches"] / max(r["steps"], 1)}

    def run_workload(name, cfg_, steps, warmup, clk, with_roofline):
        reads = sim.SimReads(cfg_)
        # replicas: every rank holds the whole read store and tables and
        # corrects its own contiguous shard of anchors, window by window
        first, count = shard.shard_range(reads.n, rank, world, bool(cfg_.paired))
        wins = [(first + s0, c) for s0, c in windows_of(count, args.window, bool(cfg_.paired))]
        runs = {}
        for form in forms_wanted:
            runs[form] = run_form(reads, cfg_, form, wins, steps, warmup, clk, digest=form in ("plain", "batched"))
            runs[form]["steps"] = steps
        forest_run = run_form(reads, cfg_, "forest", wins, 0, 0)
        forms = {f: summary(r) for f, r in runs.items()}
        forms["forest"] = {"tp": forest_run["score"]["tp"], "fp": forest_run["score"]["fp"],
                           "fn": forest_run["score"]["fn"], "driver": "plain", "timed": False}
        if "plain" in runs and "batched" in runs:
            # every flag and corrected base of every read, compared window by window
            same = runs["plain"]["res"] == runs["batched"]["res"] and runs["plain"]["score"] == runs["batched"]["score"]
            if dist is not None:
                t = torch.tensor([int(same)], dtype=torch.int64, device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.MIN)
                same = bool(t.item())
            forms["batched_bit_exact_with_plain"] = same
        bl = runs["batched_learned"]
        forms["batched_shape"] = {k: bl["st1"][k] for k in ("batch_anchors", "align_blocks", "msa_warps",
                                                          "streams", "seconds_tune")}
        out = {"reads": reads, "runs": runs, "forms": forms, "wins": wins}
        return out

    def roofline_of(plain, clk_mhz):
        p0, p1 = plain["st0"], plain["st1"]
        steps = plain["steps"]
        n_anchors = plain["anchors"]
        lmax = plain["lmax"]
        stages = {"align": p1["seconds_align"] - p0["seconds_align"],
                  "filter": p1["seconds_filter"] - p0["seconds_filter"],
                  "msa": p1["seconds_msa"] - p0["seconds_msa"],
                  "candidates": p1["seconds_candidates"] - p0["seconds_candidates"]}
        dom = max(stages, key=stages.get)
        cands = p1["unique_candidates"] - p0["unique_candidates"]
        msa_c = p1["msa_candidates"] - p0["msa_candidates"]
        raw = p1["raw_candidate_ids"] - p0["raw_candidate_ids"]
        wp = (lmax + 31) // 32 + 1
        pitch = (lmax + 15) // 16
        if dom == "align":
            kbytes = cands * (4 + 2 + 16 * wp + 8) + n_anchors * (8 * wp + 10)
            launches = p1["align_launches"] - p0["align_launches"]
            kname = "align_lane_kernel"
        elif dom == "msa":
            kbytes = msa_c * (13 + 4 * pitch) + n_anchors * (4 * pitch + 2 + lmax + 1)
            launches = p1["msa_launches"] - p0["msa_launches"]
            kname = "msa_warp_kernel"
        else:
            kbytes = raw * 4 + n_anchors * 48 * 24
            launches = max(p1["align_launches"] - p0["align_launches"], 1)
            kname = "gather_unique_kernel"
        launches = max(launches, 1)
        dur = stages[dom] / launches
        # the path's algorithmic bytes per anchor: 2-bit anchor row, 48 signature
        # keys and 48 lookup slots probed, 4 B per raw id, the unique candidates'
        # rows and lengths, the result written (flag and corrected bases); one
        # launch of the dominant kernel processes one batch of anchors
        path_bytes = n_anchors * (4 * pitch + 48 * 8 + 48 * 16 + 1 + lmax) + 4 * raw + cands * (4 * pitch + 4)
        bytes_launch = path_bytes / launches
        achieved = bytes_launch / dur / 1e9
        roof = {"bound": "hbm", "kernel": kname, "form": "plain", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": (ALIGN_DRAM_BYTES_PER_CANDIDATE * cands / launches) if dom == "align" else None,
                "peak_kind": peak_kind, "algorithmic_bytes_per_launch": bytes_launch,
                "algorithmic_bytes_per_anchor": path_bytes / max(n_anchors, 1),
                "kernel_bytes_per_launch": kbytes / launches, "avg_launch_ms": dur * 1e3,
                "stage_seconds_per_step": {k: v / max(steps, 1) for k, v in stages.items()},
                "note": "integer-issue bound, see `int`; the HBM fraction is low by construction.  traffic = "
                        "measured DRAM bytes per candidate (ncu) x candidates per launch: the kernel reads each "
                        "candidate's precomputed forward and reverse-complement hi/lo planes (96 B, in 32 B sectors) "
                        "where the algorithmic count takes its 40 B 2-bit row"}
        if dom == "align":
            # warp instructions per candidate (ncu, committed profile) x the launch's candidates,
            # over the launch's CUDA-event time, against 152 SMs x 4 schedulers x 1 instruction per
            # cycle at the median SM clock sampled during the timed region
            mhz = clk_mhz or 2070.0
            inst = ALIGN_WARP_INST_PER_CANDIDATE * cands / launches
            peak_i = 152 * 4 * mhz * 1e6
            roof["int"] = {"bound": "int-issue", "achieved": inst / dur / 1e9, "peak": peak_i / 1e9,
                           "unit": "G warp-instructions/s", "frac": inst / dur / peak_i, "sm_mhz": mhz,
                           "warp_instructions_per_candidate": ALIGN_WARP_INST_PER_CANDIDATE,
                           "alu_pipe_active_ncu": ALIGN_ALU_PIPE_ACTIVE,
                           "source": "smsp__inst_executed.sum per candidate from ncu "
                                     "(profiles/align_lane_kernel_c4_shape_20mbp.md) x candidates of an average launch"}
        return roof

    clk = ClockSampler(local, paused=True)
    with clk:
        head = run_workload(args.config, cfg, args.steps, args.warmup, clk, True)
    reads = head["reads"]
    forms = head["forms"]
    bl = head["runs"]["batched_learned"]
    value = forms["batched_learned"]["value"]
    launches = bl["st1"]["kernel_launches"] - bl["st0"]["kernel_launches"]
    clocks = clk.summary()
    roof = roofline_of(head["runs"]["plain"], clocks.get("sm_mhz")) if "plain" in head["runs"] else None

    def e2e_of(reads, cfg_, steps):
        """The metric end to end through the C ABI from pinned host memory
        (batched + learned): per step a fresh context, every read appended,
        the device build, the classifier load, the correction of this
        replica's anchors and every result copied back."""
        n = reads.n
        lmax = int(reads.lengths.max())
        flags = np.zeros(n, np.uint8)
        rows = np.zeros((n, lmax), np.uint8)
        rt = torch.cuda.cudart()
        pinned = []
        for a in (reads.sequences, reads.offsets, flags, rows):
            # page-lock the caller's buffers (untimed set-up), as a caller streaming reads would
            if int(rt.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) == 0:
                pinned.append(a)
        k = max(1, steps)
        te = 0.0
        sf, sc = shard.shard_range(n, rank, world, bool(cfg_.paired))  # this replica's anchors
        for i in range(1 + k):
            barrier()
            t0 = time.perf_counter()
            g2 = make_ctx(reads, cfg_, "batched_learned")
            g2.correct(sf, sc, flags[sf:sf + sc], rows[sf:sf + sc])
            g2.close()
            barrier()
            if i >= 1:
                te += time.perf_counter() - t0
        for a in pinned:
            rt.cudaHostUnregister(a.ctypes.data)
        te = max_over_ranks(te)
        return {"value": n * k / te, "unit": UNIT, "steps": k, "seconds_per_step": te / k,
                "h2d_bytes_per_step": int(reads.sequences.nbytes + reads.offsets.nbytes + len(model)),
                "d2h_bytes_per_step": int(flags[sf:sf + sc].nbytes + rows[sf:sf + sc].nbytes),
                "pinned": len(pinned) == 4,
                "form": "batched_learned",
                "includes": "fresh context, append of every read from pinned host memory, device read-store and "
                            "table build, classifier load, correction of every anchor (each replica its shard), "
                            "every result to pinned host memory, destroy"}

    e2e = None if args.no_e2e else e2e_of(reads, cfg, args.e2e_steps)

    def sweep_one(reads, cfg_, form, t):
        o = form_options(cfg_, form)
        o.driver = capi.CG_DRIVER_BATCHED
        o.threshold_anchor = t
        g = capi.CareGpu(o)
        g.append_reads(reads.sequences, reads.offsets)
        g.build_tables()
        if form == "batched_learned":
            g.load_classifier(model)
        else:
            g.load_forest(forest)
        flags, rows = g.correct()
        g.close()
        sc = reads.score_results(0, flags, rows)
        return {"threshold": t, "tp": sc["tp"], "fp": sc["fp"], "fn": sc["fn"]}

    def matched(curve_a, curve_b):
        """FP of curve_b at the TP of each point of curve_a (linear between
        curve_b's neighbouring thresholds; None outside its TP range)."""
        pts = sorted((p["tp"], p["fp"]) for p in curve_b)
        out = []
        for p in curve_a:
            fp = None
            for (t0, f0), (t1, f1) in zip(pts, pts[1:]):
                if t0 <= p["tp"] <= t1:
                    fp = f0 if t1 == t0 else f0 + (f1 - f0) * (p["tp"] - t0) / (t1 - t0)
                    break
            out.append({"tp": p["tp"], "fp_forest": p["fp"], "fp_learned_at_same_tp": fp,
                        "forest_threshold": p["threshold"]})
        return out

    def threshold_sweep(name):
        cfg_ = sim.CONFIGS[name]
        reads_ = sim.SimReads(cfg_)
        ts = (0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 0.95)
        forest_curve = [sweep_one(reads_, cfg_, "forest", t) for t in ts]
        learned_curve = [sweep_one(reads_, cfg_, "batched_learned", t) for t in ts]
        reads_.close()
        return {"forest": forest_curve, "learned": learned_curve, "learned_fp_at_forest_tp":
                matched(forest_curve, learned_curve),
                "forest_file": os.path.relpath(forest_path, REPO)}

    sweeps = None
    if args.sweep and args.sweep != "none":
        sweeps = {name: threshold_sweep(name) for name in args.sweep.split(",") if name}

    secondary = None
    if args.secondary and args.secondary != "none" and args.secondary != args.config:
        cfg2 = sim.CONFIGS[args.secondary]
        sec = run_workload(args.secondary, cfg2, args.steps, args.warmup, None, False)
        secondary = {"config": workload_desc(args.secondary, cfg2), "forms": sec["forms"],
                     "plain_stage_seconds_per_step":
                         roofline_of(sec["runs"]["plain"], clocks.get("sm_mhz"))["stage_seconds_per_step"]
                         if "plain" in sec["runs"] else None,
                     "e2e": None if args.no_e2e else e2e_of(sec["reads"], cfg2, max(args.e2e_steps, 5))}
        del sec

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(reads, cfg, threads)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": bl["dev"] / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": dict(workload_desc(args.config, cfg), window_anchors=args.window,
                               step="one window of anchors against the tables of the whole read set"),
                "form": "batched_learned", "forms": forms, "e2e": e2e, "gpu_launches": int(launches),
                "roofline": roof, "cpu_baseline": cpu, "clocks": clocks, "wall_seconds_timed": bl["wall"],
                "build_seconds": bl["st1"]["seconds_build"], "score": bl["score"],
                "stats": {k: bl["st1"][k] for k in ("raw_candidate_ids", "unique_candidates", "aligned_candidates",
                                                   "msa_candidates", "msa_builds", "corrected_anchors",
                                                   "hq_anchors", "table_keys", "table_values",
                                                   "learned_columns", "learned_corrections")},
                "secondary": secondary, "threshold_sweep": sweeps}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
