"""ORACLE -- test infrastructure, not product code.

ctypes front end of liboracle.so, the plain C++ restatement of the reference
CARE correction path (oracle/care_oracle.cpp).  Only tests/, the smoke check
in __graft_entry__ and bench.py's CPU-baseline leg use it, as the checker of
the GPU path; the product library neither links nor calls it.

Parity pin: tests/test_oracle_golden.py checks this restatement against
fixtures that the reference itself produced (tests/golden/, made by
tests/golden/make_golden.py from the reference built by oracle/ref.mk).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(ORACLE_DIR)
LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(ORACLE_DIR, "care_oracle.cpp")
    hdr = os.path.join(REPO_DIR, "include", "care_gpu.h")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-I" + os.path.join(REPO_DIR, "include"), src, "-o", LIB]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
    return LIB


def reference_dir() -> str:
    """Where the reference (RabbitQCPlus) source tree is looked for: the
    CARE_REFERENCE_DIR environment variable, else a directory named
    `reference` beside this repository."""
    return os.environ.get("CARE_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO_DIR), "reference")


def build_reference(ref_dir: str | None = None, jobs: int = 8) -> bool:
    """Compile the reference's own CARE sources into oracle/_ref (only where the
    reference tree exists; returns False otherwise)."""
    ref_dir = ref_dir or reference_dir()
    if not os.path.isdir(os.path.join(ref_dir, "src")):
        return False
    cmd = ["make", "-f", os.path.join("oracle", "ref.mk"), f"REF={ref_dir}", f"-j{jobs}"]
    r = subprocess.run(cmd, cwd=REPO_DIR, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout[-4000:])
    return True


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [P, P, P, P, ctypes.c_uint64, ctypes.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_info.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_double)]
        L.orc_signatures.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P]
        L.orc_candidates.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_correct.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P, P, ctypes.c_size_t, ctypes.c_int, P]
        L.orc_load_forest.argtypes = [P, P, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float]
        L.orc_check_orientation_shortcut.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, P]
        _lib = L
    return _lib


class Oracle:
    """The CPU restatement over one read set."""

    def __init__(self, options, sequences: np.ndarray, offsets: np.ndarray, qualities: np.ndarray | None,
                 threads: int = os.cpu_count() or 1):
        L = lib()
        self._L = L
        self._keep = (np.ascontiguousarray(sequences, dtype=np.uint8),
                      np.ascontiguousarray(offsets, dtype=np.uint64),
                      None if qualities is None else np.ascontiguousarray(qualities, dtype=np.uint8))
        self.options = options
        self.threads = threads
        self._h = L.orc_create(ctypes.byref(options), self._keep[0].ctypes.data, self._keep[1].ctypes.data,
                               None if self._keep[2] is None else self._keep[2].ctypes.data,
                               len(offsets) - 1, threads)
        if not self._h:
            raise ValueError("oracle: invalid input")
        n, lmax, k, nm, bs = ctypes.c_uint64(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        L.orc_info(self._h, ctypes.byref(n), ctypes.byref(lmax), ctypes.byref(k), ctypes.byref(nm), ctypes.byref(bs))
        self.n, self.max_length, self.k, self.num_maps = n.value, lmax.value, k.value, nm.value
        self.build_seconds = bs.value

    def load_forest(self, data: bytes, max_trees: int = 0xFFFFFFFF, threshold: float = 0.5):
        buf = np.frombuffer(data, np.uint8)
        if self._L.orc_load_forest(self._h, buf.ctypes.data, len(buf), max_trees, threshold) != 0:
            raise ValueError("malformed forest file")

    def signatures(self, first: int, n: int) -> np.ndarray:
        out = np.zeros((n, self.num_maps), dtype=np.uint64)
        assert self._L.orc_signatures(self._h, first, n, out.ctypes.data) == 0
        return out

    def candidates(self, anchor: int) -> np.ndarray:
        cap = 48 * 65536
        out = np.zeros(cap, dtype=np.uint32)
        cnt = ctypes.c_uint32()
        assert self._L.orc_candidates(self._h, anchor, out.ctypes.data, cap, ctypes.byref(cnt)) == 0
        return out[:cnt.value].copy()

    def check_orientation_shortcut(self, first: int, count: int, threads: int | None = None) -> dict:
        """(candidate, orientation scanned first) cases of anchors [first,
        first + count), how many the device alignment's one-plane shortcut
        decides, and how many of those the reference's rule decides otherwise
        (oracle/care_oracle.cpp: orc_check_orientation_shortcut)."""
        out = np.zeros(3, dtype=np.uint64)
        assert self._L.orc_check_orientation_shortcut(self._h, first, count, threads or self.threads,
                                                        out.ctypes.data) == 0
        return {"cases": int(out[0]), "decided": int(out[1]), "wrong": int(out[2])}

    def correct(self, first: int = 0, count: int | None = None, threads: int | None = None):
        """Returns (flags[count], corrected[count, max_length], counters[8]).  With
        candidate correction the range is the whole read set and the flags are
        combined as cg_combine_results combines them."""
        if count is None:
            count = self.n - first
        flags = np.zeros(count, dtype=np.uint8)
        seqs = np.zeros((count, max(self.max_length, 1)), dtype=np.uint8)
        counters = np.zeros(8, dtype=np.uint64)
        rc = self._L.orc_correct(self._h, first, count, flags.ctypes.data, seqs.ctypes.data, seqs.shape[1],
                                 threads or self.threads, counters.ctypes.data)
        if rc != 0:
            raise ValueError(f"oracle correct failed ({rc})")
        return flags, seqs, counters

    def close(self):
        if getattr(self, "_h", None):
            self._L.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
