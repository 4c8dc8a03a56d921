"""Make the forest classifier fixtures (run where the reference tree exists).

No trained forest ships with the reference, so this script produces one the
way the reference's own workflow implies:
  1. run the reference in Print mode (--correctionType 2) on a training read
     set; it writes the 13 anchor features of every non-HQ anchor position
     whose base differs from the consensus (include/classification.hpp:100-121,
     extract_anchor_v3 at :748-797) to anchorfeatures.txt;
  2. label each row from the generator's truth (1 = the consensus base is the
     true base), train a random forest with scikit-learn;
  3. write it in the reference's forest file format (include/forest.hpp:38-55,
     141-162: u64-length descriptor "13 extract_anchor_v3", u32 tree count,
     per tree a u32 node count and the nodes in preorder, each
     {u8 feature, f64 split, u8 flag, then lhs/rhs as f32 leaf probability or
     a nested node}; flag bit 1 = lhs is a leaf, bit 0 = rhs is a leaf);
  4. run the reference in Forest mode (--correctionType 1 --ml-forestfile) on a
     separate test read set and store its output like the other fixtures.
Outputs: forest_anchor.bin, forest_se.npz, and a "forest_se" manifest entry.

`python tests/golden/make_forest.py workload` makes the workload-scale forest
the learned classifier is compared with (forest_varlen.bin, described in
forest_varlen.json): the same Print-mode features, from the reads the learned
classifier is trained on, with the forest's size chosen on a held-out seed.
"""
from __future__ import annotations

import dataclasses
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from rabbitqcplus_gb300 import sim  # noqa: E402
import make_golden  # noqa: E402

TRAIN = sim.SimConfig(seed=201, genome_length=120_000, repeat_families=8, repeat_copies=4, num_reads=24_000,
                      read_len_min=100, read_len_max=150, sub_rate_5p=0.004, sub_rate_3p=0.03)
TEST = sim.SimConfig(seed=202, genome_length=60_000, repeat_families=4, repeat_copies=4, num_reads=12_000,
                     read_len_min=100, read_len_max=150, sub_rate_5p=0.004, sub_rate_3p=0.03)
N_TREES = 16
MAX_LEAVES = 128


def ref(*args, cwd):
    exe = os.path.join(REPO, "oracle", "_ref", "ref_care")
    r = subprocess.run([exe, *args], cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-3000:])


def serialize(forest, path):
    out = bytearray()
    desc = "13 extract_anchor_v3".encode()
    out += struct.pack("<Q", len(desc)) + desc
    out += struct.pack("<I", len(forest.estimators_))
    for est in forest.estimators_:
        t = est.tree_
        out += struct.pack("<I", t.node_count)

        def leaf_prob(i):
            v = t.value[i][0]
            return float(v[1] / v.sum()) if v.sum() > 0 else 0.0

        def node(i):
            l, r = t.children_left[i], t.children_right[i]
            l_leaf = t.children_left[l] == -1
            r_leaf = t.children_left[r] == -1
            flag = (2 if l_leaf else 0) | (1 if r_leaf else 0)
            b = struct.pack("<BdB", int(t.feature[i]), float(t.threshold[i]), flag)
            b += struct.pack("<f", leaf_prob(l)) if l_leaf else node(l)
            b += struct.pack("<f", leaf_prob(r)) if r_leaf else node(r)
            return b

        if t.children_left[0] == -1:
            raise RuntimeError("degenerate tree")
        out += node(0)
    with open(path, "wb") as f:
        f.write(bytes(out))


def main():
    from sklearn.ensemble import RandomForestClassifier
    import oracle
    oracle.build_reference()
    with tempfile.TemporaryDirectory() as work:
        tr = sim.SimReads(TRAIN)
        tr.write_fastq(os.path.join(work, "train.fq"))
        ref("-i", "train.fq", "-o", "train_out.fq", "-d", work, "-c", "30", "-k", "20", "-t", "8", "--print",
            cwd=work)
        rows, labels = [], []
        with open(os.path.join(work, "anchorfeatures.txt")) as f:
            header = f.readline().strip()
            assert header == "13 extract_anchor_v3", header
            for line in f:
                t = line.split()
                rid, pos, cons = int(t[0]), int(t[1]), t[2]
                truth = chr(tr.truth[tr.offsets[rid] + pos])
                rows.append([float(x) for x in t[3:16]])
                labels.append(1 if cons == truth else 0)
        X = np.array(rows, np.float32)
        y = np.array(labels, np.int32)
        print("training rows", len(y), "positive", int(y.sum()))
        clf = RandomForestClassifier(n_estimators=N_TREES, max_leaf_nodes=MAX_LEAVES, random_state=7, n_jobs=8)
        clf.fit(X, y)
        fpath = os.path.join(HERE, "forest_anchor.bin")
        serialize(clf, fpath)
        te = sim.SimReads(TEST)
        te.write_fastq(os.path.join(work, "test.fq"))
        ref("-i", "test.fq", "-o", "test_out.fq", "-d", work, "-c", "30", "-k", "20", "-t", "8", "--forest", fpath,
            cwd=work)
        outs = make_golden.fastq_sequences(os.path.join(work, "test_out.fq"), te.n)
        out_all = np.frombuffer(b"".join(outs), dtype=np.uint8)
        diff = np.nonzero(out_all != te.sequences)[0]
        rid = (np.searchsorted(te.offsets, diff, side="right") - 1).astype(np.uint32)
        pos = (diff - te.offsets[rid]).astype(np.uint16)
        np.savez_compressed(os.path.join(HERE, "forest_se.npz"),
                            read=np.diff(rid, prepend=np.uint32(0)).astype(np.uint32), pos=pos, base=out_all[diff])
        # the same read set in Classic mode, for the TP/FP comparison
        ref("-i", "test.fq", "-o", "test_classic.fq", "-d", work, "-c", "30", "-k", "20", "-t", "8", cwd=work)
        classic = np.frombuffer(b"".join(make_golden.fastq_sequences(os.path.join(work, "test_classic.fq"), te.n)),
                                dtype=np.uint8)
        mpath = os.path.join(HERE, "manifest.json")
        manifest = json.load(open(mpath))
        manifest["forest_se"] = {
            "config": dataclasses.asdict(TEST), "options": {"coverage": 30, "k": 20, "forest": "forest_anchor.bin"},
            "num_reads": te.n, "input_md5": make_golden.md5(te.sequences.tobytes()),
            "input_qual_md5": make_golden.md5(te.qualities.tobytes()),
            "output_md5": make_golden.md5(out_all.tobytes()), "changed_reads": int(len(np.unique(rid))),
            "score": te.score(out_all), "classic_score": te.score(classic),
            "forest": {"trees": N_TREES, "max_leaf_nodes": MAX_LEAVES, "training_rows": int(len(y)),
                       "train_config": dataclasses.asdict(TRAIN)}}
        with open(mpath, "w") as f:
            json.dump(manifest, f, indent=1, sort_keys=True)
        print("forest", manifest["forest_se"]["score"], "classic", manifest["forest_se"]["classic_score"])


def print_dump(reads: sim.SimReads, work: str, name: str):
    """The reference's Print-mode features of a read set, labelled from the truth."""
    fq = os.path.join(work, f"{name}.fq")
    reads.write_fastq(fq)
    d = os.path.join(work, name)
    os.makedirs(d, exist_ok=True)
    cov = round(reads.cfg.num_reads * (reads.cfg.read_len_min + reads.cfg.read_len_max) / 2 /
                reads.cfg.genome_length)
    ref("-i", fq, "-o", "out.fq", "-d", d, "-c", str(cov), "-k", "20", "-t", str(os.cpu_count() or 8), "--print",
        cwd=d)
    X = []
    rid, pos, cons = [], [], []
    with open(os.path.join(d, "anchorfeatures.txt")) as f:
        header = f.readline().strip()
        assert header == "13 extract_anchor_v3", header
        for line in f:
            t = line.split()
            rid.append(int(t[0]))
            pos.append(int(t[1]))
            cons.append(ord(t[2]))
            X.append([float(x) for x in t[3:16]])
    rid = np.array(rid, np.int64)
    idx = reads.offsets.astype(np.int64)[rid] + np.array(pos, np.int64)
    y = (reads.truth[idx] == np.array(cons, np.uint8)).astype(np.int32)
    return np.array(X, np.float32), y


def workload_forest(seeds=(1001, 1002, 1003), validation_seed=1004, genome=10_000_000):
    """The forest the learned decision is compared with: trained on the
    reference's Print-mode features of the reads the learned classifier was
    trained on (10 Mbp genome with repeats, reads U[50,250] at 30x, generator
    seeds 1001-1003), its size chosen by the log-loss on a held-out seed.
    Writes forest_varlen.bin and the "forest_varlen" manifest entry."""
    from sklearn.ensemble import RandomForestClassifier
    from sklearn.metrics import log_loss
    import oracle
    oracle.build_reference()
    with tempfile.TemporaryDirectory() as work:
        Xs, ys = [], []
        for seed in seeds:
            r = sim.SimReads(sim.scaled("c3_10mbp_varlen", genome, seed=seed))
            X, y = print_dump(r, work, f"train{seed}")
            print(f"seed {seed}: {len(y)} columns, {y.mean():.4f} positive", flush=True)
            Xs.append(X)
            ys.append(y)
            r.close()
        X, y = np.concatenate(Xs), np.concatenate(ys)
        rv = sim.SimReads(sim.scaled("c3_10mbp_varlen", genome, seed=validation_seed))
        Xv, yv = print_dump(rv, work, "validation")
    rng = np.random.default_rng(5)
    sub = rng.choice(len(y), size=min(len(y), 1_500_000), replace=False)
    grid = []
    for leaves in (256, 1024, 4096, 16384):
        clf = RandomForestClassifier(n_estimators=32, max_leaf_nodes=leaves, random_state=7,
                                     n_jobs=os.cpu_count() or 8)
        clf.fit(X[sub], y[sub])
        loss = float(log_loss(yv, np.clip(clf.predict_proba(Xv)[:, 1], 1e-6, 1 - 1e-6)))
        grid.append({"trees": 32, "max_leaf_nodes": leaves, "validation_log_loss": loss})
        print(grid[-1], flush=True)
    best = min(grid, key=lambda g: g["validation_log_loss"])
    clf = RandomForestClassifier(n_estimators=64, max_leaf_nodes=best["max_leaf_nodes"], random_state=7,
                                 n_jobs=os.cpu_count() or 8)
    clf.fit(X, y)
    loss = float(log_loss(yv, np.clip(clf.predict_proba(Xv)[:, 1], 1e-6, 1 - 1e-6)))
    fpath = os.path.join(HERE, "forest_varlen.bin")
    serialize(clf, fpath)
    mpath = os.path.join(HERE, "forest_varlen.json")
    with open(mpath, "w") as f:
        json.dump({"trees": 64, "max_leaf_nodes": best["max_leaf_nodes"], "training_rows": int(len(y)),
                   "positive": float(y.mean()), "train_seeds": list(seeds), "validation_seed": validation_seed,
                   "genome": genome, "grid": grid, "validation_log_loss": loss,
                   "bytes": os.path.getsize(fpath)}, f, indent=1)
    print("forest_varlen", best, loss, os.path.getsize(fpath), flush=True)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "workload":
        workload_forest()
    else:
        main()
