"""Failure paths of the device engine, provoked from the host or with short
device waits -- never by a GPU fault:

* the learned decision's tensor-core waits given 0 polls
  (cg_set_classifier_wait_limit): every inference block gives up on its first
  tile, drains its MMAs at the full limit and frees its tensor memory; the
  call returns CG_ERR_TIMEOUT, the columns keep the fallback (classic)
  decision, cg_stats counts the blocks, and with the default limit restored
  the same context gives the normal result again;
* a simulated out-of-memory (cg_set_allocation_fault): the call fails with
  CG_ERR_OUT_OF_MEMORY after the block cache was emptied, nothing leaks, and
  the library works afterwards;
* a truncated FASTQ through the device file path and an output directory that
  cannot be created: CG_ERR_IO, no partial result.
"""
import os

import numpy as np
import pytest

from oracle import mlp
from rabbitqcplus_gb300 import capi, learned, sim

pytestmark = pytest.mark.gpu


def small_reads(seed=71):
    cfg = sim.SimConfig(seed=seed, genome_length=40_000, repeat_families=3, repeat_copies=3, num_reads=8_000,
                        sub_rate_5p=0.004, sub_rate_3p=0.03)
    return sim.SimReads(cfg)


def ctx(reads, **kw):
    g = capi.CareGpu(capi.CareOptions.defaults(30.0, **kw))
    g.append_reads(reads.sequences, reads.offsets)
    g.build_tables()
    return g


def correct_into(g, n, lmax):
    flags = np.zeros(n, np.uint8)
    out = np.zeros((n, lmax), np.uint8)
    rc = g._L.cg_correct(g._h, 0, n, flags.ctypes.data, out.ctypes.data, lmax)
    return rc, flags, out


def same_results(reads, a, b):
    fa, oa = a
    fb, ob = b
    assert np.array_equal(fa, fb)
    for i in np.nonzero(fa & capi.CG_RESULT_CORRECTED)[0]:
        L = reads.lengths[i]
        assert np.array_equal(oa[i, :L], ob[i, :L]), f"anchor {i}"


def test_classifier_logits_timeout_and_recovery():
    m = mlp.random_model(3)
    x = np.random.default_rng(2).uniform(0, 1, (1000, mlp.F)).astype(np.float32)
    try:
        capi.set_classifier_wait_limit(0)
        with pytest.raises(capi.CareError, match="timeout"):
            capi.classifier_logits(mlp.serialize(m), x)
    finally:
        capi.set_classifier_wait_limit(-1)
    z = capi.classifier_logits(mlp.serialize(m), x)
    zo, _, _, _ = mlp.forward(m, x)
    assert np.all(np.abs(z - zo) <= 1e-2 + 1e-2 * np.abs(zo))


@pytest.mark.parametrize("driver", [capi.CG_DRIVER_PLAIN, capi.CG_DRIVER_BATCHED])
def test_correction_timeout_reports_and_keeps_fallback(driver):
    r = small_reads()
    model = open(learned.DEFAULT_MODEL, "rb").read()
    shape = dict(driver=driver, batch_anchors=2048, align_blocks=152, msa_warps=4, streams=2)
    classic = ctx(r, **shape)
    n, lmax = classic.read_info()
    rc, cf, co = correct_into(classic, n, lmax)
    assert rc == capi.CG_OK
    classic.close()
    g = ctx(r, correction_type=capi.CG_CORR_LEARNED, **shape)
    g.load_classifier(model)
    rc, lf, lo = correct_into(g, n, lmax)
    assert rc == capi.CG_OK
    assert g.stats()["learned_corrections"] > 0
    try:
        capi.set_classifier_wait_limit(0)
        rc, tf, to = correct_into(g, n, lmax)
    finally:
        capi.set_classifier_wait_limit(-1)
    assert rc == capi.CG_ERR_TIMEOUT
    assert "timed out" in g._L.cg_last_error(g._h).decode()
    st = g.stats()
    assert st["classifier_timeouts"] > 0
    # no block scored a column: every decision is the fallback's, i.e. the classic one
    same_results(r, (tf, to), (cf, co))
    # the context keeps working with the default limit
    rc, lf2, lo2 = correct_into(g, n, lmax)
    assert rc == capi.CG_OK
    same_results(r, (lf2, lo2), (lf, lo))
    assert g.stats()["classifier_timeouts"] == st["classifier_timeouts"]
    g.close()


def test_out_of_memory_empties_cache_and_leaks_nothing():
    torch = pytest.importorskip("torch")
    r = sim.SimReads(sim.scaled("c0_1mbp_se", 400_000))
    capi.release_cached_memory(-1)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    g = ctx(r)
    ref = g.correct()
    g.close()  # its blocks go to the cache
    free1, _ = torch.cuda.mem_get_info()
    assert free1 < free0
    for after in (0, 3, 8):
        made = []
        try:
            capi.set_allocation_fault(after)
            with pytest.raises(capi.CareError, match="out of memory"):
                g = capi.CareGpu(capi.CareOptions.defaults(30.0))
                made.append(g)
                g.append_reads(r.sequences, r.offsets)
                g.build_tables()
                g.correct()
        finally:
            capi.set_allocation_fault(-1)
        # the failing request emptied the cache (the failed context holds a few blocks at most)
        free2, _ = torch.cuda.mem_get_info()
        assert free2 > free1
        for g in made:
            g.close()
    capi.release_cached_memory(-1)
    free3, _ = torch.cuda.mem_get_info()
    assert abs(free3 - free0) <= 64 << 20, (free0, free3)
    g = ctx(r)
    out = g.correct()
    g.close()
    same_results(r, out, ref)
    capi.release_cached_memory(-1)


def test_truncated_fastq_through_device_path_is_an_io_error(tmp_path):
    r = small_reads(72)
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    data = open(fq, "rb").read()
    cut = data.rfind(b"\n+\n")  # the last record loses its quality line
    with open(fq, "wb") as f:
        f.write(data[:cut + 3])
    os.makedirs(tmp_path / "out")
    o = capi.CareOptions.defaults(30.0)
    o.host_file_io = 0
    with pytest.raises(capi.CareError, match="I/O"):
        capi.correct_files(o, [fq], str(tmp_path / "out"), ["o.fq"])


def test_output_directory_that_cannot_exist_is_an_io_error(tmp_path):
    r = small_reads(73)
    fq = str(tmp_path / "in.fq")
    r.write_fastq(fq)
    blocker = tmp_path / "file"
    blocker.write_text("x")
    o = capi.CareOptions.defaults(30.0)
    with pytest.raises(capi.CareError, match="I/O"):
        capi.correct_files(o, [fq], str(blocker / "sub"), ["o.fq"])
    assert not os.path.exists(str(blocker / "sub"))


def test_bad_offsets_are_refused_at_the_first_bad_read():
    """cg_append_reads checks every read's offsets before any copy (the check
    runs on several host threads for large appends): the first read, in read
    order, whose offsets descend or that is longer than CG_MAX_READ_LENGTH is
    named; the context takes a valid append afterwards."""
    n = 300_000
    offs = np.arange(n + 1, dtype=np.uint64) * 100
    seqs = np.full(int(offs[-1]) + 10_000, ord("A"), np.uint8)
    down = offs.copy()
    down[200_002] = down[200_001] - 1    # read 200001 descends
    down[250_001:] += 2000               # read 250000 is too long, after it
    longf = offs.copy()
    longf[100_001:] += 2000              # read 100000 is too long
    longf[250_002] = longf[250_001] - 1  # a descent after it
    g = capi.CareGpu(capi.CareOptions.defaults(30.0))
    with pytest.raises(capi.CareError, match="offsets not ascending at 200001"):
        g.append_reads(seqs, down)
    with pytest.raises(capi.CareError, match="read 100000 longer than 1024"):
        g.append_reads(seqs, longf)
    r = small_reads(74)
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    n_, lmax = g.read_info()
    assert n_ == r.n and lmax == int(r.lengths.max())
    flags, _ = g.correct()
    assert int((flags & capi.CG_RESULT_CORRECTED).astype(bool).sum()) > r.n // 4
    g.close()
