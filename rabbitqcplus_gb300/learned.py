"""Learned correction classifier: training data, training and evaluation.

The learned decision (correction_type CG_CORR_LEARNED) scores every MSA
column of a non-high-quality anchor whose consensus differs from the anchor's
base with a 32-64-64-1 MLP and takes the consensus where the output reaches
the threshold (0.5); elsewhere the classic rule decides.  The network is
trained on the device (cg_train_classifier) on columns whose label comes from
the generator's truth: 1 when the consensus base is the read's true base.

    python -m rabbitqcplus_gb300.learned train --out model.bin
    python -m rabbitqcplus_gb300.learned evaluate --model model.bin

Training data default: reads shaped like the variable-length workload (10 Mbp
genome with repeats, reads U[50,250] at 30x) from generator seeds that the
evaluation does not use, until at least 5M labelled columns are collected.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from . import capi, sim

DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "classifier_varlen.bin")
TRAIN_SEEDS = (1001, 1002, 1003, 1004, 1005, 1006, 1007, 1008)
EVAL_SEED = 17  # the workload's own seed


def options(reads: sim.SimReads, correction_type: int, **kw) -> capi.CareOptions:
    cfg = reads.cfg
    cov = round(cfg.num_reads * (cfg.read_len_min + cfg.read_len_max) / 2 / cfg.genome_length)
    o = capi.CareOptions.defaults(float(cov), kmerlength=20, correction_type=correction_type,
                                  pair_mode=capi.CG_PAIR_PE if cfg.paired else capi.CG_PAIR_SE)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def collect(reads: sim.SimReads, **kw):
    """Columns of the learned decision with their truth labels, in (anchor, position) order.

    The device records columns in an unspecified order; sorting them makes a
    training run (minibatch order drawn from its seed) reproducible.
    """
    g = capi.CareGpu(options(reads, capi.CG_CORR_LEARNED, **kw))
    g.append_reads(reads.sequences, reads.offsets)
    g.build_tables()
    feats, anchors, pos, cons = g.columns()
    g.close()
    order = np.lexsort((pos, anchors))
    feats, anchors, pos, cons = feats[order], anchors[order], pos[order], cons[order]
    idx = reads.offsets.astype(np.int64)[anchors.astype(np.int64)] + pos.astype(np.int64)
    labels = (reads.truth[idx] == cons).astype(np.uint8)
    return feats, labels


def training_set(min_columns: int = 5_000_000, genome: int = 10_000_000, seeds=TRAIN_SEEDS, log=print):
    fs, ls = [], []
    total = 0
    for seed in seeds:
        cfg = sim.scaled("c3_10mbp_varlen", genome, seed=seed)
        r = sim.SimReads(cfg)
        f, y = collect(r)
        r.close()
        fs.append(f)
        ls.append(y)
        total += len(f)
        log(f"seed {seed}: {len(f)} columns ({y.mean():.3f} positive), total {total}")
        if total >= min_columns:
            break
    return np.concatenate(fs), np.concatenate(ls)


def correct(reads: sim.SimReads, correction_type: int, model: bytes | None = None, forest: bytes | None = None,
            **kw):
    g = capi.CareGpu(options(reads, correction_type, **kw))
    g.append_reads(reads.sequences, reads.offsets)
    g.build_tables()
    if model is not None:
        g.load_classifier(model)
    if forest is not None:
        g.load_forest(forest)
    flags, seqs = g.correct()
    st = g.stats()
    g.close()
    out = capi.apply_corrections(reads.sequences, reads.offsets, flags, seqs)
    return reads.score(out), st, flags, seqs


def evaluate(reads: sim.SimReads, model: bytes, forest: bytes | None = None, **kw) -> dict:
    """TP/FP/FN of the classic rule, the learned decision and (if given) the forest."""
    res = {}
    res["classic"], _, _, _ = correct(reads, capi.CG_CORR_CLASSIC, **kw)
    res["learned"], st, _, _ = correct(reads, capi.CG_CORR_LEARNED, model=model, **kw)
    res["learned"]["columns"] = st["learned_columns"]
    res["learned"]["taken"] = st["learned_corrections"]
    res["learned"]["overflow"] = st["learned_overflow"]
    if forest is not None:
        res["forest"], _, _, _ = correct(reads, capi.CG_CORR_FOREST, forest=forest, **kw)
    return res


def log_loss(model: bytes, f: np.ndarray, y: np.ndarray) -> float:
    """Mean binary cross-entropy of a classifier's outputs (the inference kernel's logits)."""
    z = capi.classifier_logits(model, f).astype(np.float64)
    return float(np.mean(np.logaddexp(0.0, z) - y * z))


def score_threshold(reads: sim.SimReads, correction_type: int, t: float, model: bytes | None = None,
                    forest: bytes | None = None) -> dict:
    """TP/FP/FN of a decision at threshold_anchor t (batched driver)."""
    g = capi.CareGpu(options(reads, correction_type, threshold_anchor=t, driver=capi.CG_DRIVER_BATCHED))
    g.append_reads(reads.sequences, reads.offsets)
    g.build_tables()
    if model is not None:
        g.load_classifier(model)
    if forest is not None:
        g.load_forest(forest)
    flags, rows = g.correct()
    g.close()
    sc = reads.score_results(0, flags, rows)
    return {"threshold": t, "tp": sc["tp"], "fp": sc["fp"], "fn": sc["fn"]}


def fp_at_tp(curve: list, tp: int):
    """FP of a (tp, fp) curve at `tp`, linear between its points; None outside."""
    pts = sorted((p["tp"], p["fp"]) for p in curve)
    for (t0, f0), (t1, f1) in zip(pts, pts[1:]):
        if t0 <= tp <= t1:
            return f0 if t1 == t0 else f0 + (f1 - f0) * (tp - t0) / (t1 - t0)
    return None


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--columns", type=int, default=5_000_000)
    t.add_argument("--genome", type=int, default=10_000_000)
    t.add_argument("--grid", default="4:2e-3,8:1e-3,16:1e-3,16:5e-4,24:1e-3,32:7e-4,16:1e-3:2,16:1e-3:3",
                   help="epochs:learning-rate[:seed] settings; the one with the lowest validation loss is kept")
    t.add_argument("--batch", type=int, default=4096)
    t.add_argument("--seed", type=int, default=1)
    t.add_argument("--validation-seed", type=int, default=1004)
    e = sub.add_parser("evaluate")
    e.add_argument("--model", default=DEFAULT_MODEL)
    e.add_argument("--forest", default=None)
    e.add_argument("--genome", type=int, default=10_000_000)
    w = sub.add_parser("sweep", help="TP/FP of the learned decision and a forest over thresholds")
    w.add_argument("--model", default=DEFAULT_MODEL)
    w.add_argument("--forest", required=True)
    w.add_argument("--workloads", default="c1_10mbp_repeats_se,c3_10mbp_varlen")
    args = ap.parse_args(argv)
    if args.cmd == "train":
        t0 = time.time()
        f, y = training_set(args.columns, args.genome, log=lambda m: print(m, file=sys.stderr))
        rv = sim.SimReads(sim.scaled("c3_10mbp_varlen", args.genome, seed=args.validation_seed))
        fv, yv = collect(rv)
        rv.close()
        t1 = time.time()
        runs = []
        best = None
        for item in args.grid.split(","):
            parts = item.split(":")
            ep, lr = int(parts[0]), float(parts[1])
            seed = int(parts[2]) if len(parts) > 2 else args.seed
            o = capi.TrainOptions.defaults(epochs=ep, batch_rows=args.batch, learning_rate=lr, seed=seed)
            model, losses = capi.train_classifier(f, y, o)
            vl = log_loss(model, fv, yv)
            runs.append({"epochs": ep, "learning_rate": lr, "seed": seed, "steps": int(len(losses)),
                         "train_loss_last_epoch": float(losses[-max(len(losses) // ep, 1):].mean()),
                         "validation_loss": vl})
            if best is None or vl < best[0]:
                best = (vl, model, runs[-1])
        t2 = time.time()
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        with open(args.out, "wb") as fh:
            fh.write(best[1])
        print(json.dumps({"columns": int(len(f)), "positive": float(y.mean()), "validation_columns": int(len(fv)),
                          "validation_seed": args.validation_seed, "grid": runs, "chosen": best[2],
                          "collect_s": t1 - t0, "train_s": t2 - t1, "out": args.out}))
    elif args.cmd == "sweep":
        with open(args.model, "rb") as fh:
            model = fh.read()
        with open(args.forest, "rb") as fh:
            forest = fh.read()
        ts = (0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 0.95)
        out = {}
        for name in args.workloads.split(","):
            r = sim.SimReads(sim.CONFIGS[name])
            fc = [score_threshold(r, capi.CG_CORR_FOREST, x, forest=forest) for x in ts]
            lc = [score_threshold(r, capi.CG_CORR_LEARNED, x, model=model) for x in ts]
            r.close()
            out[name] = {"forest": fc, "learned": lc,
                         "learned_fp_at_forest_tp": [{"tp": p["tp"], "fp_forest": p["fp"],
                                                      "fp_learned": fp_at_tp(lc, p["tp"])} for p in fc]}
        print(json.dumps(out))
    else:
        with open(args.model, "rb") as fh:
            model = fh.read()
        forest = None
        if args.forest:
            with open(args.forest, "rb") as fh:
                forest = fh.read()
        r = sim.SimReads(sim.scaled("c3_10mbp_varlen", args.genome, seed=EVAL_SEED))
        print(json.dumps(evaluate(r, model, forest)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
