"""Locates, builds and loads the in-tree shared libraries.

libcaregpu.so is the product: hand-written sm_103a CUDA kernels plus the
C ABI declared in include/care_gpu.h.  libcaresim.so is the seeded workload
generator.  Both are built in-tree (rabbitqcplus_gb300/lib/) by build(); the
product path never falls back to anything else: if libcaregpu.so is missing
or fails to load, loading raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "lib")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# Host code is compiled as ISO C++17 with floating-point contraction off so
# that float thresholds computed on the host round exactly as the reference's.
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
# Device code: no fused multiply-add contraction, IEEE division and sqrt
# (the correction path's float arithmetic must round exactly as the reference).
NVCCFLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
             "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp",
             "--expt-relaxed-constexpr", "-I" + INCLUDE_DIR, "-I" + CSRC]

GPU_CU_SOURCES = [
    "k_store.cu",
    "k_tables.cu",
    "k_sort.cu",
    "k_correct.cu",
    "k_learned.cu",
    "care_capi.cu",
    "care_train.cu",
    "care_files.cu",
]
GPU_CPP_SOURCES = [
    "host/seqio.cpp",
    "host/care_host.cpp",
]
# gzip FASTA/FASTQ through zlib where its header is installed
HAVE_ZLIB = os.path.exists("/usr/include/zlib.h")

_lock = threading.Lock()
_loaded: dict[str, ctypes.CDLL] = {}


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _headers() -> list[str]:
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh", ".hpp"))]
    out += [os.path.join(INCLUDE_DIR, f) for f in os.listdir(INCLUDE_DIR) if f.endswith(".h")]
    return out


def build_sim(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(CSRC, "sim", "care_sim.cpp")
    out = os.path.join(LIB_DIR, "libcaresim.so")
    if force or _newer(out, [src, os.path.join(CSRC, "sim", "care_sim.h")]):
        _run([CXX, *CXXFLAGS, "-shared", src, "-o", out])
    return out


def build_gpu(force: bool = False, jobs: int = 8) -> str:
    os.makedirs(os.path.join(LIB_DIR, "obj"), exist_ok=True)
    out = os.path.join(LIB_DIR, "libcaregpu.so")
    hdrs = _headers()
    objs, cmds = [], []
    for s in GPU_CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(LIB_DIR, "obj", os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            cmds.append([NVCC, *NVCCFLAGS, "-c", src, "-o", obj])
    for s in GPU_CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(LIB_DIR, "obj", os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            cmds.append([CXX, *CXXFLAGS, *(["-DCG_HAVE_ZLIB"] if HAVE_ZLIB else []), "-I" + INCLUDE_DIR, "-I" + CSRC,
                         "-I/usr/local/cuda/include", "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    if force or cmds or not os.path.exists(out):
        _run([NVCC, ARCH, "-shared", *objs, "-o", out, "-Xcompiler", "-fopenmp", "-lcudart", "-lgomp",
              *(["-lz"] if HAVE_ZLIB else [])])
    return out


def _load(name: str, builder) -> ctypes.CDLL:
    with _lock:
        if name in _loaded:
            return _loaded[name]
        path = os.path.join(LIB_DIR, name)
        if not os.path.exists(path):
            builder()
        lib = ctypes.CDLL(path)
        _loaded[name] = lib
        return lib


def sim() -> ctypes.CDLL:
    lib = _load("libcaresim.so", build_sim)
    if not getattr(lib, "_typed", False):
        P = ctypes.c_void_p
        lib.cgsim_create.restype = P
        lib.cgsim_create.argtypes = [P]
        lib.cgsim_destroy.argtypes = [P]
        lib.cgsim_num_reads.restype = ctypes.c_uint64
        lib.cgsim_num_reads.argtypes = [P]
        lib.cgsim_total_bases.restype = ctypes.c_uint64
        lib.cgsim_total_bases.argtypes = [P]
        lib.cgsim_offsets.restype = ctypes.POINTER(ctypes.c_uint64)
        lib.cgsim_offsets.argtypes = [P]
        for f in ("cgsim_sequences", "cgsim_qualities", "cgsim_truth"):
            getattr(lib, f).restype = ctypes.c_void_p
            getattr(lib, f).argtypes = [P]
        lib.cgsim_indel_flags.restype = ctypes.c_void_p
        lib.cgsim_indel_flags.argtypes = [P]
        lib.cgsim_write_fastq.restype = ctypes.c_int
        lib.cgsim_write_fastq.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p]
        lib.cgsim_score.argtypes = [P, ctypes.c_char_p] + [ctypes.POINTER(ctypes.c_uint64)] * 4
        lib.cgsim_score_results.argtypes = [P, ctypes.c_uint64, ctypes.c_uint64, P, P, ctypes.c_uint64] + \
            [ctypes.POINTER(ctypes.c_uint64)] * 4
        lib._typed = True
    return lib


def gpu() -> ctypes.CDLL:
    """The product library.  Raises if it cannot be built or loaded."""
    return _load("libcaregpu.so", build_gpu)
