"""Helpers shared by the tests: golden-fixture loading and input re-creation."""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys

import numpy as np

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
GOLDEN = os.path.join(TESTS, "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from rabbitqcplus_gb300 import sim, capi  # noqa: E402


def manifest() -> dict:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def case_names() -> list[str]:
    return sorted(manifest().keys())


def options_for(entry: dict) -> capi.CareOptions:
    o = entry["options"]
    return capi.CareOptions.defaults(
        float(o["coverage"]), kmerlength=int(o["k"]), num_hash_functions=int(o.get("maps", 48)),
        use_quality_scores=int(bool(o.get("quality"))),
        exclude_ambiguous_reads=int(bool(o.get("exclude_ambiguous"))),
        pair_mode=capi.CG_PAIR_PE if o.get("paired") else capi.CG_PAIR_SE,
        correction_type=capi.CG_CORR_FOREST if o.get("forest") else capi.CG_CORR_CLASSIC,
        correct_candidates=int(bool(o.get("candidates"))),
        new_columns_to_correct=int(o.get("new_columns", 15)),
        quality_score_bits=int(o.get("quality_bits", 8)),
        fixed_number_of_reads=int(o.get("fixed_reads", 0)))


def forest_bytes(entry: dict) -> bytes | None:
    name = entry["options"].get("forest")
    if not name:
        return None
    with open(os.path.join(GOLDEN, name), "rb") as f:
        return f.read()


def reads_for(entry: dict) -> sim.SimReads:
    cfg = sim.SimConfig(**entry["config"])
    return sim.SimReads(cfg)


def md5(a: np.ndarray) -> str:
    return hashlib.md5(np.ascontiguousarray(a).tobytes()).hexdigest()


def expected_output(name: str, reads: sim.SimReads) -> np.ndarray:
    """The reference's output read bases, rebuilt from the stored edit list."""
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    rid = np.cumsum(z["read"].astype(np.uint64))
    pos = z["pos"].astype(np.uint64)
    out = reads.sequences.copy()
    out[reads.offsets[rid] + pos] = z["base"]
    return out


def load_stages(name: str) -> dict:
    """Parse a reference stage dump (oracle/ref_stages.cpp output)."""
    path = os.path.join(GOLDEN, f"{name}.stages.txt.gz")
    sigs, anchors = {}, []
    cur = None
    with gzip.open(path, "rt") as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "SIG":
                sigs[int(t[1])] = [int(x, 16) for x in t[2:]]
            elif t[0] == "ANCHOR":
                cur = {"id": int(t[1]), "len": int(t[3]), "aln": [], "w": []}
                anchors.append(cur)
            elif t[0] == "CAND":
                cur["cand"] = [int(x) for x in t[2:]]
            elif t[0] == "ALN":
                cur["aln"].append([int(x) for x in t[1:]])
            elif t[0] == "KEPT":
                cur["kept"] = [int(x) for x in t[2:]]
            elif t[0] == "W":
                cur["w"].append((int(t[1]), int(t[2]), int(t[3], 16)))
            elif t[0] == "MSA":
                cur["msa"] = [int(x) for x in t[1:]]
            elif t[0] == "CONS":
                cur["cons"] = t[1]
            elif t[0] == "SUP":
                cur["sup"] = [int(x, 16) for x in t[1:]]
            elif t[0] == "COV":
                cur["cov"] = [int(x) for x in t[1:]]
            elif t[0] == "PROP":
                cur["prop"] = [int(t[1], 16), int(t[2], 16), int(t[3]), int(t[4]), int(t[5])]
            elif t[0] == "CORR":
                cur["corr"] = (int(t[1]), t[2])
    return {"sigs": sigs, "anchors": anchors}
