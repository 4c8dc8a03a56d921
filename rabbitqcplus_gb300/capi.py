"""ctypes mirror of include/care_gpu.h and a thin Python front end.

`CareOptions` is the C struct `cg_options`; `CareGpu` owns one `cg_ctx`.
The calls go straight to libcaregpu.so; there is no Python or CPU fallback: a
missing library or a failing CUDA call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib

CG_OK = 0
CG_ERR_INVALID_ARGUMENT, CG_ERR_UNSUPPORTED, CG_ERR_CUDA, CG_ERR_OUT_OF_MEMORY = 1, 2, 3, 4
CG_ERR_STATE, CG_ERR_IO, CG_ERR_TIMEOUT = 5, 6, 7
CG_ERRORS = {1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "out of memory", 5: "bad state",
             6: "I/O error", 7: "timeout"}
CG_MAX_HASHMAPS = 48
CG_PAIR_SE, CG_PAIR_PE = 0, 1
CG_CORR_CLASSIC, CG_CORR_FOREST, CG_CORR_PRINT, CG_CORR_LEARNED = 0, 1, 2, 3
CG_RESULT_CORRECTED, CG_RESULT_HQ = 1, 2
CG_RESULT_CANDIDATES, CG_RESULT_REJECTED, CG_RESULT_CANDIDATE_RECORD = 4, 8, 16
CG_DRIVER_PLAIN, CG_DRIVER_BATCHED = 0, 1


class CareOptions(ctypes.Structure):
    _fields_ = [
        ("kmerlength", ctypes.c_int32),
        ("num_hash_functions", ctypes.c_int32),
        ("estimated_coverage", ctypes.c_float),
        ("estimated_errorrate", ctypes.c_float),
        ("m_coverage", ctypes.c_float),
        ("max_error_rate", ctypes.c_float),
        ("min_overlap_ratio", ctypes.c_float),
        ("min_overlap", ctypes.c_int32),
        ("paired_filter_threshold", ctypes.c_float),
        ("new_columns_to_correct", ctypes.c_int32),
        ("use_quality_scores", ctypes.c_int32),
        ("exclude_ambiguous_reads", ctypes.c_int32),
        ("correct_candidates", ctypes.c_int32),
        ("pair_mode", ctypes.c_int32),
        ("correction_type", ctypes.c_int32),
        ("threshold_anchor", ctypes.c_float),
        ("device", ctypes.c_int32),
        ("batch_anchors", ctypes.c_int32),
        ("driver", ctypes.c_int32),
        ("align_blocks", ctypes.c_int32),
        ("msa_warps", ctypes.c_int32),
        ("streams", ctypes.c_int32),
        ("host_file_io", ctypes.c_int32),
        ("quality_score_bits", ctypes.c_int32),
        ("fixed_number_of_reads", ctypes.c_uint32),
        ("reserved0", ctypes.c_int32),
        ("hashtable_memory_bytes", ctypes.c_uint64),
    ]

    @classmethod
    def defaults(cls, coverage: float = 30.0, **kw) -> "CareOptions":
        """Reference defaults (include/options.hpp:36-99) with --coverage set."""
        o = cls()
        o.kmerlength = 20
        o.num_hash_functions = 48
        o.estimated_coverage = coverage
        o.estimated_errorrate = 0.06
        o.m_coverage = 0.6
        o.max_error_rate = 0.2
        o.min_overlap_ratio = 0.3
        o.min_overlap = 30
        o.paired_filter_threshold = 0.06
        o.new_columns_to_correct = 15
        o.use_quality_scores = 0
        o.exclude_ambiguous_reads = 0
        o.correct_candidates = 0
        o.pair_mode = CG_PAIR_SE
        o.correction_type = CG_CORR_CLASSIC
        o.threshold_anchor = 0.5
        o.quality_score_bits = 8
        o.device = 0
        o.batch_anchors = 0
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class CgStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "num_reads", "num_anchors_processed", "raw_candidate_ids", "unique_candidates", "aligned_candidates",
        "msa_candidates", "msa_builds", "corrected_anchors", "hq_anchors", "table_keys", "table_values")] + [
        ("kmerlength", ctypes.c_int32), ("num_maps", ctypes.c_int32), ("max_read_length", ctypes.c_int32),
        ("reserved", ctypes.c_int32), ("seconds_build", ctypes.c_double), ("seconds_correct", ctypes.c_double),
        ("seconds_candidates", ctypes.c_double), ("seconds_align", ctypes.c_double), ("seconds_msa", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64), ("align_launches", ctypes.c_uint64), ("msa_launches", ctypes.c_uint64),
        ("seconds_filter", ctypes.c_double), ("batch_anchors", ctypes.c_int32), ("align_blocks", ctypes.c_int32),
        ("msa_warps", ctypes.c_int32), ("streams", ctypes.c_int32), ("seconds_tune", ctypes.c_double),
        ("graph_replays", ctypes.c_uint64), ("learned_columns", ctypes.c_uint64),
        ("learned_corrections", ctypes.c_uint64), ("learned_overflow", ctypes.c_uint64),
        ("candidate_corrections", ctypes.c_uint64), ("classifier_timeouts", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


# every symbol include/care_gpu.h declares
EXPORTED = ["cg_default_options", "cg_create", "cg_destroy", "cg_last_error", "cg_append_reads",
            "cg_build_tables", "cg_correct", "cg_get_stats", "cg_get_read_info", "cg_get_signatures",
            "cg_get_candidates", "cg_correct_files", "cg_load_forest", "cg_get_candidates_noalloc",
            "cg_classifier_size", "cg_load_classifier", "cg_get_columns", "cg_default_train_options",
            "cg_train_classifier", "cg_classifier_gradients", "cg_classifier_logits", "cg_release_cached_memory",
            "cg_combine_results", "cg_set_classifier_wait_limit", "cg_set_allocation_fault"]
CLASSIFIER_FEATURES = 32
CLASSIFIER_PARAMS = 6337  # w1 64x32, w2 64x64, w3 64, b1 64, b2 64, b3


class TrainOptions(ctypes.Structure):
    """cg_train_options (include/care_gpu.h)."""
    _fields_ = [
        ("device", ctypes.c_int32),
        ("epochs", ctypes.c_int32),
        ("batch_rows", ctypes.c_int32),
        ("learning_rate", ctypes.c_float),
        ("seed", ctypes.c_uint32),
        ("reserved0", ctypes.c_int32),
        ("init_model", ctypes.c_void_p),
        ("init_model_size", ctypes.c_size_t),
        ("reserved", ctypes.c_int32 * 8),
    ]

    @classmethod
    def defaults(cls, **kw) -> "TrainOptions":
        o = cls()
        gpu_lib().cg_default_train_options(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o


def gpu_lib() -> ctypes.CDLL:
    L = _lib.gpu()
    if not getattr(L, "_cg_typed", False):
        P = ctypes.c_void_p
        L.cg_default_options.argtypes = [P]
        L.cg_create.argtypes = [P, ctypes.POINTER(P)]
        L.cg_destroy.argtypes = [P]
        L.cg_last_error.restype = ctypes.c_char_p
        L.cg_last_error.argtypes = [P]
        L.cg_append_reads.argtypes = [P, P, P, P, ctypes.c_uint64]
        L.cg_build_tables.argtypes = [P]
        L.cg_correct.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P, P, ctypes.c_size_t]
        L.cg_get_stats.argtypes = [P, P]
        L.cg_combine_results.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P, ctypes.POINTER(ctypes.c_uint64)]
        L.cg_get_read_info.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)]
        L.cg_get_signatures.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P]
        L.cg_get_candidates.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        L.cg_correct_files.argtypes = [P, P, ctypes.c_int, ctypes.c_char_p, P, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
        L.cg_load_forest.argtypes = [P, P, ctypes.c_size_t, ctypes.c_uint32]
        L.cg_get_candidates_noalloc.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32,
                                                ctypes.POINTER(ctypes.c_uint32)]
        L.cg_classifier_size.restype = ctypes.c_size_t
        L.cg_classifier_size.argtypes = []
        L.cg_load_classifier.argtypes = [P, P, ctypes.c_size_t]
        L.cg_get_columns.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P, P, P, P, ctypes.c_uint64,
                                     ctypes.POINTER(ctypes.c_uint64)]
        L.cg_default_train_options.argtypes = [P]
        L.cg_train_classifier.argtypes = [P, P, P, ctypes.c_uint64, P, ctypes.c_size_t, P, ctypes.c_uint64,
                                          ctypes.POINTER(ctypes.c_uint64)]
        L.cg_classifier_gradients.argtypes = [ctypes.c_int, P, ctypes.c_size_t, P, P, ctypes.c_uint32, P,
                                              ctypes.POINTER(ctypes.c_float)]
        L.cg_classifier_logits.argtypes = [ctypes.c_int, P, ctypes.c_size_t, P, ctypes.c_uint64, P]
        L.cg_release_cached_memory.argtypes = [ctypes.c_int]
        L.cg_set_classifier_wait_limit.argtypes = [ctypes.c_int, ctypes.c_int64]
        L.cg_set_allocation_fault.argtypes = [ctypes.c_int64]
        for f in EXPORTED:
            if f not in ("cg_destroy", "cg_default_options", "cg_last_error", "cg_classifier_size",
                         "cg_default_train_options"):
                getattr(L, f).restype = ctypes.c_int
        L._cg_typed = True
    return L


class CareError(RuntimeError):
    pass


def set_allocation_fault(after: int) -> None:
    """Every device-memory request after the next `after` fails as out of memory (< 0: off)."""
    gpu_lib().cg_set_allocation_fault(after)


def release_cached_memory(device: int = -1) -> None:
    rc = gpu_lib().cg_release_cached_memory(device)
    if rc != CG_OK:
        raise CareError(f"cg_release_cached_memory: {CG_ERRORS.get(rc, rc)}")


def set_classifier_wait_limit(polls: int, device: int = 0) -> None:
    """Polls of the classifier's per-tile MMA waits on `device` (< 0: the default)."""
    rc = gpu_lib().cg_set_classifier_wait_limit(device, polls)
    if rc != CG_OK:
        raise CareError(f"cg_set_classifier_wait_limit: {CG_ERRORS.get(rc, rc)}")


class CareGpu:
    """One device context: append reads, build tables, correct anchors."""

    def __init__(self, options: CareOptions):
        self._L = gpu_lib()
        self.options = options
        h = ctypes.c_void_p()
        rc = self._L.cg_create(ctypes.byref(options), ctypes.byref(h))
        if rc != CG_OK:
            raise CareError(f"cg_create failed: {CG_ERRORS.get(rc, rc)}")
        self._h = h

    def _check(self, rc: int, what: str):
        if rc != CG_OK:
            msg = self._L.cg_last_error(self._h).decode(errors="replace")
            raise CareError(f"{what}: {CG_ERRORS.get(rc, rc)}: {msg}")

    def append_reads(self, sequences: np.ndarray, offsets: np.ndarray, qualities: np.ndarray | None = None):
        s = np.ascontiguousarray(sequences, dtype=np.uint8)
        o = np.ascontiguousarray(offsets, dtype=np.uint64)
        q = None if qualities is None else np.ascontiguousarray(qualities, dtype=np.uint8)
        self._check(self._L.cg_append_reads(self._h, s.ctypes.data, o.ctypes.data,
                                            None if q is None else q.ctypes.data, len(o) - 1), "cg_append_reads")

    def build_tables(self):
        self._check(self._L.cg_build_tables(self._h), "cg_build_tables")

    def load_forest(self, data: bytes, max_trees: int = 0):
        buf = np.frombuffer(data, np.uint8)
        self._check(self._L.cg_load_forest(self._h, buf.ctypes.data, len(buf), max_trees), "cg_load_forest")

    def read_info(self):
        n, l = ctypes.c_uint64(), ctypes.c_int32()
        self._check(self._L.cg_get_read_info(self._h, ctypes.byref(n), ctypes.byref(l)), "cg_get_read_info")
        return n.value, l.value

    def correct(self, first: int = 0, count: int | None = None, flags: np.ndarray | None = None,
                out: np.ndarray | None = None, combine: bool | None = None):
        """cg_correct over [first, first + count).  With candidate correction and
        a call that covers every read, the flags also go through
        cg_combine_results (combine=False keeps cg_correct's flags)."""
        n, lmax = self.read_info()
        if count is None:
            count = n - first
        if flags is None:
            flags = np.zeros(count, dtype=np.uint8)
        if out is None:
            out = np.zeros((count, max(lmax, 1)), dtype=np.uint8)
        self._check(self._L.cg_correct(self._h, first, count, flags.ctypes.data, out.ctypes.data, out.strides[0]),
                    "cg_correct")
        if combine is None:
            combine = bool(self.options.correct_candidates) and first == 0 and count == n
        if combine:
            self.combine(0, flags)
        return flags, out

    def combine(self, first: int, flags: np.ndarray) -> int:
        """cg_combine_results on flags of reads [first, first + len(flags)), in
        place; returns the number of saved candidate records among them."""
        flags = np.ascontiguousarray(flags, dtype=np.uint8)
        recs = ctypes.c_uint64()
        self._check(self._L.cg_combine_results(self._h, first, len(flags), flags.ctypes.data, ctypes.byref(recs)),
                    "cg_combine_results")
        return recs.value

    def stats(self) -> dict:
        s = CgStats()
        self._check(self._L.cg_get_stats(self._h, ctypes.byref(s)), "cg_get_stats")
        return s.as_dict()

    def signatures(self, first: int, n: int, num_maps: int) -> np.ndarray:
        out = np.zeros((n, num_maps), dtype=np.uint64)
        self._check(self._L.cg_get_signatures(self._h, first, n, out.ctypes.data), "cg_get_signatures")
        return out

    def candidates(self, anchor: int) -> np.ndarray:
        cap = 48 * 65536
        out = np.zeros(cap, dtype=np.uint32)
        cnt = ctypes.c_uint32()
        self._check(self._L.cg_get_candidates(self._h, anchor, out.ctypes.data, cap, ctypes.byref(cnt)),
                    "cg_get_candidates")
        return out[:cnt.value].copy()

    def candidates_noalloc(self, anchor: int, out: np.ndarray) -> int:
        """cg_get_candidates_noalloc into a caller-owned uint32 array; returns the count."""
        assert out.dtype == np.uint32 and out.flags["C_CONTIGUOUS"]
        cnt = ctypes.c_uint32()
        self._check(self._L.cg_get_candidates_noalloc(self._h, anchor, out.ctypes.data, out.size, ctypes.byref(cnt)),
                    "cg_get_candidates_noalloc")
        return cnt.value

    def load_classifier(self, data: bytes):
        buf = np.frombuffer(data, np.uint8)
        self._check(self._L.cg_load_classifier(self._h, buf.ctypes.data, len(buf)), "cg_load_classifier")

    def columns(self, first: int = 0, count: int | None = None):
        """Columns the learned decision scores: (features[k][32], anchor ids, positions, consensus bases)."""
        n, _ = self.read_info()
        if count is None:
            count = n - first
        k = ctypes.c_uint64()
        rc = self._L.cg_get_columns(self._h, first, count, None, None, None, None, 0, ctypes.byref(k))
        if rc not in (CG_OK, 1):
            self._check(rc, "cg_get_columns")
        cap = k.value
        f = np.zeros((max(cap, 1), CLASSIFIER_FEATURES), np.float32)
        a = np.zeros(max(cap, 1), np.uint64)
        p = np.zeros(max(cap, 1), np.uint16)
        c = np.zeros(max(cap, 1), np.uint8)
        self._check(self._L.cg_get_columns(self._h, first, count, f.ctypes.data, a.ctypes.data, p.ctypes.data,
                                           c.ctypes.data, cap, ctypes.byref(k)), "cg_get_columns")
        m = k.value
        return f[:m], a[:m], p[:m], c[:m]

    def close(self):
        if getattr(self, "_h", None):
            self._L.cg_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def apply_corrections(sequences: np.ndarray, offsets: np.ndarray, flags: np.ndarray,
                      corrected: np.ndarray) -> np.ndarray:
    """Output reads as the reference's STEP3 writes them
    (src/correctionresultoutput.cpp:1256-1551): a read with an anchor
    correction becomes its corrected sequence unless the combine step rejected
    it (CG_RESULT_REJECTED); others stay unchanged."""
    out = np.array(sequences, dtype=np.uint8, copy=True)
    lens = np.diff(offsets).astype(np.int64)
    idx = np.nonzero(((flags & CG_RESULT_CORRECTED) != 0) & ((flags & CG_RESULT_REJECTED) == 0))[0]
    for i in idx:
        b = int(offsets[i])
        out[b:b + lens[i]] = corrected[i, :lens[i]]
    return out


def correct_files(options: CareOptions, inputs: list[str], output_directory: str, outputs: list[str],
                  quality_labels: bool = False, gz_output: bool = False) -> int:
    """File-to-file correction (care::performCorrection); returns the number of correction records."""
    L = gpu_lib()
    ins = (ctypes.c_char_p * len(inputs))(*[x.encode() for x in inputs])
    outs = (ctypes.c_char_p * len(outputs))(*[x.encode() for x in outputs])
    n = ctypes.c_uint64()
    rc = L.cg_correct_files(ctypes.byref(options), ctypes.cast(ins, ctypes.c_void_p), len(inputs),
                            output_directory.encode(), ctypes.cast(outs, ctypes.c_void_p), len(outputs),
                            int(quality_labels), int(gz_output), ctypes.byref(n))
    if rc != CG_OK:
        raise CareError(f"cg_correct_files: {CG_ERRORS.get(rc, rc)}")
    return n.value


def _model_buf(model: bytes):
    return np.frombuffer(model, np.uint8)


def train_classifier(features: np.ndarray, labels: np.ndarray, options: TrainOptions | None = None,
                     init_model: bytes | None = None):
    """Train the learned classifier on the device; returns (serialized model, per-step losses)."""
    L = gpu_lib()
    o = options or TrainOptions.defaults()
    f = np.ascontiguousarray(features, np.float32)
    y = np.ascontiguousarray(labels, np.uint8)
    assert f.ndim == 2 and f.shape[1] == CLASSIFIER_FEATURES and len(y) == len(f)
    init = None
    if init_model is not None:
        init = _model_buf(init_model)
        o.init_model = init.ctypes.data
        o.init_model_size = len(init)
    size = L.cg_classifier_size()
    out = np.zeros(size, np.uint8)
    steps_max = (len(f) // max(o.batch_rows, 1)) * o.epochs
    losses = np.zeros(max(steps_max, 1), np.float32)
    steps = ctypes.c_uint64()
    rc = L.cg_train_classifier(ctypes.byref(o), f.ctypes.data, y.ctypes.data, len(f), out.ctypes.data, size,
                               losses.ctypes.data, len(losses), ctypes.byref(steps))
    if rc != CG_OK:
        raise CareError(f"cg_train_classifier: {CG_ERRORS.get(rc, rc)}")
    return out.tobytes(), losses[:steps.value].copy()


def classifier_gradients(model: bytes, features: np.ndarray, labels: np.ndarray, device: int = 0):
    """Mean loss and its gradient (6337 values) computed by the training kernels."""
    L = gpu_lib()
    m = _model_buf(model)
    f = np.ascontiguousarray(features, np.float32)
    y = np.ascontiguousarray(labels, np.uint8)
    g = np.zeros(CLASSIFIER_PARAMS, np.float32)
    loss = ctypes.c_float()
    rc = L.cg_classifier_gradients(device, m.ctypes.data, len(m), f.ctypes.data, y.ctypes.data, len(f),
                                   g.ctypes.data, ctypes.byref(loss))
    if rc != CG_OK:
        raise CareError(f"cg_classifier_gradients: {CG_ERRORS.get(rc, rc)}")
    return loss.value, g


def classifier_logits(model: bytes, features: np.ndarray, device: int = 0) -> np.ndarray:
    L = gpu_lib()
    m = _model_buf(model)
    f = np.ascontiguousarray(features, np.float32)
    out = np.zeros(len(f), np.float32)
    rc = L.cg_classifier_logits(device, m.ctypes.data, len(m), f.ctypes.data, len(f), out.ctypes.data)
    if rc != CG_OK:
        raise CareError(f"cg_classifier_logits: {CG_ERRORS.get(rc, rc)}")
    return out
