"""Seeded synthetic CARE workloads (ctypes front end of libcaresim.so).

The generator itself is C++ (csrc/sim/care_sim.cpp): integer-only random
draws keyed by (seed, stream, index), so a config gives the same reads on
x86-64 and aarch64 and for any thread count.  The named configs below are the
workloads the correction path is measured and parity-tested on: a 1 Mbp
genome at 30x (200k single-end reads), a 10 Mbp genome with 200 diverged repeat
copies at 30x (2M reads, 5'->3' rising error), a paired-end 100 Mbp genome, a
variable-length workload and a 500 Mbp genome.  Scaled-down variants keep the
shape (coverage, error model, repeat density) at sizes a CPU finishes quickly.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field, asdict

import numpy as np

from . import _lib


class _Config(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("genome_length", ctypes.c_uint64),
        ("repeat_families", ctypes.c_uint32),
        ("repeat_copies", ctypes.c_uint32),
        ("repeat_min_len", ctypes.c_uint32),
        ("repeat_max_len", ctypes.c_uint32),
        ("repeat_divergence", ctypes.c_double),
        ("num_reads", ctypes.c_uint64),
        ("read_len_min", ctypes.c_uint32),
        ("read_len_max", ctypes.c_uint32),
        ("paired", ctypes.c_int32),
        ("insert_mean", ctypes.c_int32),
        ("insert_sd", ctypes.c_int32),
        ("qual_mean", ctypes.c_int32),
        ("sub_rate_5p", ctypes.c_double),
        ("sub_rate_3p", ctypes.c_double),
        ("indel_rate", ctypes.c_double),
        ("n_read_fraction", ctypes.c_double),
        ("qual_sd", ctypes.c_int32),
        ("qual_min", ctypes.c_int32),
        ("qual_max", ctypes.c_int32),
        ("err_qual_min", ctypes.c_int32),
        ("err_qual_max", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


@dataclass
class SimConfig:
    seed: int = 7
    genome_length: int = 1_000_000
    repeat_families: int = 0
    repeat_copies: int = 0
    repeat_min_len: int = 1000
    repeat_max_len: int = 5000
    repeat_divergence: float = 0.02
    num_reads: int = 200_000
    read_len_min: int = 150
    read_len_max: int = 150
    paired: bool = False
    insert_mean: int = 300
    insert_sd: int = 30
    sub_rate_5p: float = 0.01
    sub_rate_3p: float = 0.01
    indel_rate: float = 0.0
    n_read_fraction: float = 0.0
    qual_mean: int = 34
    qual_sd: int = 4
    qual_min: int = 2
    qual_max: int = 41
    err_qual_min: int = 2
    err_qual_max: int = 20

    def to_c(self) -> _Config:
        c = _Config()
        for k, v in asdict(self).items():
            setattr(c, k, int(v) if isinstance(v, bool) else v)
        return c


def _reads_for(genome: int, length: int, coverage: float, paired: bool = False) -> int:
    n = int(round(genome * coverage / length))
    if paired and n % 2:
        n += 1
    return n


# Workload shapes (sizes, coverage, error model, repeat density).
CONFIGS = {
    # 1 Mbp uniform genome, 200k x 150 bp SE reads at 30x, 1% i.i.d. substitutions
    "c0_1mbp_se": SimConfig(seed=7, genome_length=1_000_000, num_reads=200_000),
    # 10 Mbp genome + 200 diverged repeat copies (1-5 kbp, 2%), 2M x 150 bp at 30x,
    # substitution rate rising 0.2% -> 2% from 5' to 3'
    "c1_10mbp_repeats_se": SimConfig(seed=11, genome_length=10_000_000, repeat_families=40,
                                     repeat_copies=5, num_reads=2_000_000,
                                     sub_rate_5p=0.002, sub_rate_3p=0.02),
    # 100 Mbp genome with 1% repeat content, 10M pairs 2x150 bp, insert N(300,30),
    # 1% substitutions + 0.01% indels
    "c2_100mbp_pe": SimConfig(seed=13, genome_length=100_000_000, repeat_families=330,
                              repeat_copies=1, num_reads=20_000_000, paired=True,
                              sub_rate_5p=0.01, sub_rate_3p=0.01, indel_rate=0.0001),
    # as c1 with read lengths ~ U[50, 250]
    "c3_10mbp_varlen": SimConfig(seed=17, genome_length=10_000_000, repeat_families=40,
                                 repeat_copies=5, num_reads=2_000_000, read_len_min=50,
                                 read_len_max=250, sub_rate_5p=0.002, sub_rate_3p=0.02),
    # 500 Mbp genome with 5% repeat content, 100M x 150 bp, 1% substitutions
    "c4_500mbp_se": SimConfig(seed=19, genome_length=500_000_000, repeat_families=8300,
                              repeat_copies=1, num_reads=100_000_000),
}


def scaled(name: str, genome_length: int, seed: int | None = None, **kw) -> SimConfig:
    """Same shape as CONFIGS[name] at a smaller genome (same coverage)."""
    base = CONFIGS[name]
    d = asdict(base)
    frac = genome_length / base.genome_length
    d["genome_length"] = genome_length
    mean_len = (base.read_len_min + base.read_len_max) / 2
    cov = base.num_reads * mean_len / base.genome_length
    d["num_reads"] = _reads_for(genome_length, mean_len, cov, base.paired)
    if base.repeat_families:
        d["repeat_families"] = max(1, int(round(base.repeat_families * frac)))
    if seed is not None:
        d["seed"] = seed
    d.update(kw)
    return SimConfig(**d)


class SimReads:
    """Generated reads held by the C++ generator."""

    def __init__(self, cfg: SimConfig):
        lib = _lib.sim()
        self._lib = lib
        self.cfg = cfg
        c = cfg.to_c()
        self._h = lib.cgsim_create(ctypes.byref(c))
        if not self._h:
            raise ValueError(f"invalid simulation config: {cfg}")
        self.n = int(lib.cgsim_num_reads(self._h))
        tot = int(lib.cgsim_total_bases(self._h))
        self.offsets = np.ctypeslib.as_array(lib.cgsim_offsets(self._h), shape=(self.n + 1,)).copy()
        self._tot = tot
        self.sequences = self._copy(lib.cgsim_sequences)
        self._qualities = None
        self._truth = None
        self.lengths = np.diff(self.offsets).astype(np.int32)

    def _copy(self, getter) -> np.ndarray:
        if not self._h:
            raise ValueError("the generated read set was closed")
        return np.ctypeslib.as_array(ctypes.cast(getter(self._h), ctypes.POINTER(ctypes.c_uint8)),
                                     shape=(self._tot,)).copy()

    # copied on first use: a 100M-read set holds 15 GB per array
    @property
    def qualities(self) -> np.ndarray:
        if self._qualities is None:
            self._qualities = self._copy(self._lib.cgsim_qualities)
        return self._qualities

    @property
    def truth(self) -> np.ndarray:
        if self._truth is None:
            self._truth = self._copy(self._lib.cgsim_truth)
        return self._truth

    def write_fastq(self, path1: str, path2: str | None = None) -> None:
        rc = self._lib.cgsim_write_fastq(self._h, path1.encode(), path2.encode() if path2 else None)
        if rc != 0:
            raise OSError(f"cannot write {path1}")

    def score(self, corrected: np.ndarray) -> dict:
        """Base-level TP/FP/FN of corrected reads (same concatenation as input)."""
        corrected = np.ascontiguousarray(corrected, dtype=np.uint8)
        assert corrected.shape == self.sequences.shape
        tp, fp, fn, r = (ctypes.c_uint64() for _ in range(4))
        self._lib.cgsim_score(self._h, corrected.ctypes.data_as(ctypes.c_char_p), ctypes.byref(tp),
                              ctypes.byref(fp), ctypes.byref(fn), ctypes.byref(r))
        return {"tp": tp.value, "fp": fp.value, "fn": fn.value, "reads_scored": r.value}

    def score_results(self, first: int, flags: np.ndarray, rows: np.ndarray) -> dict:
        """score() of reads [first, first + len(flags)) from correction results:
        rows[j] is read first + j's corrected sequence where flags[j] says it
        was corrected (and not rejected by the combine step)."""
        flags = np.ascontiguousarray(flags, dtype=np.uint8)
        assert rows.ndim == 2 and rows.shape[0] >= len(flags) and rows.strides[1] == 1
        tp, fp, fn, r = (ctypes.c_uint64() for _ in range(4))
        self._lib.cgsim_score_results(self._h, first, len(flags), flags.ctypes.data, rows.ctypes.data,
                                      rows.strides[0], ctypes.byref(tp), ctypes.byref(fp), ctypes.byref(fn),
                                      ctypes.byref(r))
        return {"tp": tp.value, "fp": fp.value, "fn": fn.value, "reads_scored": r.value}

    def read(self, i: int) -> str:
        return self.sequences[self.offsets[i]:self.offsets[i + 1]].tobytes().decode()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cgsim_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
