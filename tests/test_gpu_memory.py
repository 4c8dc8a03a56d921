"""Device blocks released by a context are cached for the next one and given
back by cg_release_cached_memory; results do not depend on where buffers come
from."""
import numpy as np
import pytest

from rabbitqcplus_gb300 import capi, sim

pytestmark = pytest.mark.gpu


def reads():
    cfg = sim.SimConfig(seed=51, genome_length=40_000, num_reads=8_000, sub_rate_5p=0.002, sub_rate_3p=0.02)
    return sim.SimReads(cfg)


def correct_once(r):
    g = capi.CareGpu(capi.CareOptions.defaults(30.0))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    flags, out = g.correct()
    g.close()
    return flags, out


def test_cached_blocks_reused_and_released():
    torch = pytest.importorskip("torch")
    r = reads()
    lib = capi.gpu_lib()
    assert lib.cg_release_cached_memory(-1) == capi.CG_OK
    free0, _ = torch.cuda.mem_get_info()
    f1, o1 = correct_once(r)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 < free0  # the destroyed context's blocks stay cached
    f2, o2 = correct_once(r)  # served from the cache
    assert np.array_equal(f1, f2) and np.array_equal(o1, o2)
    assert lib.cg_release_cached_memory(0) == capi.CG_OK
    free2, _ = torch.cuda.mem_get_info()
    assert free2 > free1
    f3, o3 = correct_once(r)  # fresh allocations again
    assert np.array_equal(f1, f3) and np.array_equal(o1, o3)
    assert lib.cg_release_cached_memory(-1) == capi.CG_OK
