"""CPU-only checks of the boundary and host logic (no GPU needed)."""
import ctypes
import os
import re
import socket

import numpy as np
import pytest

import fixtures as fx
import oracle
from rabbitqcplus_gb300 import _lib, capi, shard, sim

INCLUDE = os.path.join(fx.REPO, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            text = open(os.path.join(INCLUDE, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(cg_\w+)\s*\(", text, flags=re.M))
    return names


def test_library_loads_and_exports_every_declared_symbol():
    L = _lib.gpu()
    decl = declared_functions()
    assert decl, "no declarations found"
    assert set(capi.EXPORTED) <= decl
    missing = [n for n in sorted(decl) if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_default_options_match_reference_defaults():
    L = capi.gpu_lib()
    o = capi.CareOptions()
    L.cg_default_options(ctypes.byref(o))
    ref = capi.CareOptions.defaults(1.0)
    for name, _ in capi.CareOptions._fields_:
        if name == "reserved":
            continue
        assert getattr(o, name) == pytest.approx(getattr(ref, name)), name


def test_context_creation_fails_loudly_without_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.CareError):
        capi.CareGpu(capi.CareOptions.defaults(30.0))


def test_invalid_options_are_rejected_before_touching_the_device():
    L = capi.gpu_lib()
    h = ctypes.c_void_p()
    for kw in ({"num_hash_functions": 0}, {"num_hash_functions": 49}, {"kmerlength": 33},
               {"estimated_coverage": 0.0}, {"pair_mode": 7}):
        o = capi.CareOptions.defaults(30.0, **kw)
        assert L.cg_create(ctypes.byref(o), ctypes.byref(h)) == 1, kw  # CG_ERR_INVALID_ARGUMENT
    for kw in ({"correct_candidates": 1, "new_columns_to_correct": 257},
               {"correct_candidates": 1, "new_columns_to_correct": -1}, {"correction_type": capi.CG_CORR_PRINT}):
        o = capi.CareOptions.defaults(30.0, **kw)
        assert L.cg_create(ctypes.byref(o), ctypes.byref(h)) == 2, kw  # CG_ERR_UNSUPPORTED


@pytest.mark.parametrize("n,world,paired", [(10, 3, False), (1000, 4, False), (7, 8, False), (100, 3, True),
                                            (2, 4, True)])
def test_shard_ranges_cover_all_anchors_once(n, world, paired):
    seen = []
    for r in range(world):
        f, c = shard.shard_range(n, r, world, paired)
        if paired:
            assert f % 2 == 0 and c % 2 == 0 or r == world - 1
        seen.extend(range(f, f + c))
    assert seen == list(range(n))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = sim.SimConfig(seed=77, genome_length=20_000, num_reads=4_000)
    r = sim.SimReads(cfg)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None, threads=2)
    f, c = shard.shard_range(r.n, rank, world)
    flags, seqs, _ = orc.correct(f, c)
    parts = [None] * world
    dist.all_gather_object(parts, (f, flags, seqs))
    if rank == 0:
        q.put(parts)
    dist.destroy_process_group()


def test_two_rank_sharded_correction_equals_single_run():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cfg = sim.SimConfig(seed=77, genome_length=20_000, num_reads=4_000)
    r = sim.SimReads(cfg)
    orc = oracle.Oracle(capi.CareOptions.defaults(30.0), r.sequences, r.offsets, None, threads=2)
    flags, seqs, _ = orc.correct()
    parts.sort(key=lambda x: x[0])
    assert np.array_equal(np.concatenate([p[1] for p in parts]), flags)
    assert np.array_equal(np.concatenate([p[2] for p in parts]), seqs)


def test_apply_corrections_only_touches_corrected_reads():
    seqs = np.frombuffer(b"AAAACCCCGGGG", np.uint8)
    offs = np.array([0, 4, 8, 12], np.uint64)
    flags = np.array([0, 1, 3], np.uint8)
    corr = np.frombuffer(b"TTTTTTTTACGA", np.uint8).reshape(3, 4)
    out = capi.apply_corrections(seqs, offs, flags, corr)
    assert out.tobytes() == b"AAAATTTTACGA"


def test_file_errors_are_reported_before_any_device_work(tmp_path):
    """cg_correct_files opens its outputs and parses host-path inputs before it
    touches the GPU: an output directory that cannot exist and a truncated
    FASTQ record both return CG_ERR_IO (runs without a GPU)."""
    r = sim.SimReads(sim.SimConfig(seed=74, genome_length=20_000, num_reads=2_000))
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    blocker = tmp_path / "file"
    blocker.write_text("x")
    o = capi.CareOptions.defaults(30.0)
    with pytest.raises(capi.CareError, match="I/O"):
        capi.correct_files(o, [fq], str(blocker / "sub"), ["o.fq"])
    data = open(fq, "rb").read()
    with open(fq, "wb") as f:
        f.write(data[:data.rfind(b"\n+\n") + 3])  # the last record loses its quality line
    os.makedirs(tmp_path / "out")
    o.host_file_io = 1
    with pytest.raises(capi.CareError, match="I/O"):
        capi.correct_files(o, [fq], str(tmp_path / "out"), ["o.fq"])
