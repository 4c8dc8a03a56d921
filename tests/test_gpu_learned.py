"""GPU tests of the learned classifier: the tensor-core kernels against the
CPU oracle (oracle/mlp.py), training, and the learned correction decision.

Tolerances: the device and the oracle round to BF16 at the same points and
accumulate in FP32, but in a different order, so a hidden activation close to
a BF16 rounding boundary can land one BF16 step apart.  Logits must agree to
1e-2 absolute (plus 1e-2 relative); gradients to 2e-2 in relative L2 norm per
parameter tensor, with the loss to 1e-5 relative.
"""
import numpy as np
import pytest

from oracle import mlp
from rabbitqcplus_gb300 import capi, learned, sim

pytestmark = pytest.mark.gpu

TENSORS = (("w1", 0, mlp.H * mlp.F), ("w2", mlp.H * mlp.F, mlp.H * mlp.H),
           ("w3", mlp.H * mlp.F + mlp.H * mlp.H, mlp.H))


def features(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (n, mlp.F)).astype(np.float32)
    x[:, 14:22] = (x[:, 14:22] > 0.7)  # one-hot-like columns
    return x


@pytest.mark.parametrize("n", [1, 15, 16, 1000, 4099])
def test_logits_match_oracle(n):
    m = mlp.random_model(11)
    x = features(n, n)
    z = capi.classifier_logits(mlp.serialize(m), x)
    zo, _, _, _ = mlp.forward(m, x)
    assert np.all(np.abs(z - zo) <= 1e-2 + 1e-2 * np.abs(zo)), float(np.abs(z - zo).max())


@pytest.mark.parametrize("n", [16, 333, 4096])
def test_gradients_match_oracle(n):
    m = mlp.random_model(12)
    x = features(n, 100 + n)
    rng = np.random.default_rng(n)
    y = rng.integers(0, 2, n).astype(np.uint8)
    loss, g = capi.classifier_gradients(mlp.serialize(m), x, y)
    lo, go = mlp.gradients(m, x, y)
    assert abs(loss - lo) <= 1e-5 * abs(lo)
    off = mlp.H * mlp.F + mlp.H * mlp.H + mlp.H
    parts = TENSORS + (("b1", off, mlp.H), ("b2", off + mlp.H, mlp.H), ("b3", off + 2 * mlp.H, 1))
    for name, i, k in parts:
        d, o = g[i:i + k], go[i:i + k]
        rel = np.linalg.norm(d - o) / max(np.linalg.norm(o), 1e-12)
        assert rel < 2e-2, (name, rel)


def test_training_learns_a_rule_and_is_deterministic():
    n = 65536
    x = features(n, 5)
    y = ((x[:, 0] + x[:, 3] > 1.0) ^ (x[:, 14] > 0.5)).astype(np.uint8)
    o = capi.TrainOptions.defaults(epochs=6, batch_rows=1024, learning_rate=3e-3, seed=9)
    model, losses = capi.train_classifier(x, y, o)
    assert len(losses) == 6 * (n // 1024)
    first, last = losses[:64].mean(), losses[-64:].mean()
    assert last < 0.5 * first, (first, last)
    z = capi.classifier_logits(model, x)
    acc = float(((z >= 0) == (y == 1)).mean())
    assert acc > 0.95, acc
    model2, _ = capi.train_classifier(x, y, capi.TrainOptions.defaults(epochs=6, batch_rows=1024,
                                                                        learning_rate=3e-3, seed=9))
    assert model == model2


def test_training_continues_from_a_model():
    n = 8192
    x = features(n, 6)
    y = (x[:, 1] > 0.5).astype(np.uint8)
    m0 = mlp.serialize(mlp.random_model(13))
    # one minibatch = the whole set: the first step's loss is the loss of m0
    model, losses = capi.train_classifier(x, y, capi.TrainOptions.defaults(epochs=2, batch_rows=n), init_model=m0)
    lo0, _ = mlp.gradients(mlp.parse(m0), x, y)
    assert losses[0] == pytest.approx(lo0, rel=1e-4)
    assert losses[1] < losses[0]


def varlen_reads(seed, genome=400_000):
    return sim.SimReads(sim.scaled("c3_10mbp_varlen", genome, seed=seed))


def test_learned_decision_plain_and_batched_agree_and_gain_over_classic():
    tr = varlen_reads(2001)
    f, y = learned.collect(tr)
    # both labels occur (the consensus is right at most recorded columns)
    assert len(f) > 10_000 and 0 < int(y.sum()) < len(y)
    model, _ = capi.train_classifier(f, y, capi.TrainOptions.defaults(epochs=8, batch_rows=1024, seed=3))
    ev = varlen_reads(2002)
    classic, _, _, _ = learned.correct(ev, capi.CG_CORR_CLASSIC)
    lp, stp, fp_, sp = learned.correct(ev, capi.CG_CORR_LEARNED, model=model)
    lb, stb, fb, sb = learned.correct(ev, capi.CG_CORR_LEARNED, model=model, driver=capi.CG_DRIVER_BATCHED,
                                      batch_anchors=4096, msa_warps=4, streams=2)
    # identical decisions from both drivers
    assert lp == lb
    assert np.array_equal(fp_, fb)
    lens = ev.lengths
    for i in np.nonzero(fp_ & capi.CG_RESULT_CORRECTED)[0]:
        assert np.array_equal(sp[i, :lens[i]], sb[i, :lens[i]]), int(i)
    assert stp["learned_columns"] == stb["learned_columns"] > 0
    assert stp["learned_corrections"] == stb["learned_corrections"]
    assert stp["learned_overflow"] == 0
    # the classic rule is the fallback: the network only adds corrections
    assert lp["tp"] >= classic["tp"]
    # what the network gains: more errors removed net of the errors it introduces
    assert lp["tp"] - lp["fp"] > classic["tp"] - classic["fp"], (lp, classic)
    # an untrained network (random weights) does not give that gain
    rnd = mlp.serialize(mlp.random_model(99))
    lr_, _, _, _ = learned.correct(ev, capi.CG_CORR_LEARNED, model=rnd)
    assert lp["tp"] - lp["fp"] > lr_["tp"] - lr_["fp"], (lp, lr_)


def test_columns_need_learned_mode_and_classifier_checks():
    r = varlen_reads(2003, genome=100_000)
    g = capi.CareGpu(learned.options(r, capi.CG_CORR_CLASSIC))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    with pytest.raises(capi.CareError):
        g.columns()
    g.close()
    g = capi.CareGpu(learned.options(r, capi.CG_CORR_LEARNED))
    g.append_reads(r.sequences, r.offsets)
    g.build_tables()
    with pytest.raises(capi.CareError):
        g.correct()  # no classifier loaded
    with pytest.raises(capi.CareError):
        g.load_classifier(b"CGMLP001" + b"\0" * 10)
    g.close()
