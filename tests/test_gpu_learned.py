"""Learned warm start on the GPU: the tcgen05 product against exact products,
the network's forward pass and gradient against the CPU oracle
(oracle/mlp_oracle.py), training, and the network inside the step (plain
results untouched when it is off, predictions applied, samples, judge)."""
import ctypes

import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(built):
    import torch

    torch.cuda.set_device(0)
    from shapes_gb300 import _lib

    return _lib


def _bf16_rand(rng, shape, scale=1.0):
    return M.bf16(rng.normal(0, scale, shape).astype(np.float32))


@pytest.mark.parametrize("n,k", [(16, 16), (64, 16), (16, 64), (64, 64), (128, 128), (208, 128), (256, 32)])
def test_tc05_gemm_matches_exact_products(built, n, k):
    import torch

    torch.cuda.set_device(0)
    from shapes_gb300 import build as B

    lib = ctypes.CDLL(str(B.PROBE_LIB))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.shapes_probe_tc05_gemm.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, fp]
    rng = np.random.default_rng(n * 1000 + k)
    a = _bf16_rand(rng, (128, k))
    b = _bf16_rand(rng, (n, k))
    d = np.zeros((128, n), dtype=np.float32)
    st = lib.shapes_probe_tc05_gemm(a.ctypes.data_as(fp), b.ctypes.data_as(fp), n, k, d.ctypes.data_as(fp))
    assert st == 0
    want = a.astype(np.float64) @ b.astype(np.float64).T
    err = np.abs(d - want)
    assert err.max() <= 1e-5 * (np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64).T).max()


def _random_net(gpu, seed, feat, tgt):
    net = gpu.Mlp(seed)
    net.fit_normalization(feat, tgt)
    return net


def _data(seed, n):
    rng = np.random.default_rng(seed)
    feat = (rng.normal(0, 1, (n, 16)) * rng.uniform(0.1, 10, 16) + rng.normal(0, 3, 16)).astype(np.float32)
    tgt = np.stack([np.maximum(feat[:, 5], 0) * 0.5 + 0.1 * feat[:, 2],
                    np.tanh(feat[:, 6]) * np.abs(feat[:, 7])], 1).astype(np.float32)
    return feat, tgt


def test_mlp_forward_matches_oracle(gpu):
    feat, tgt = _data(5, 1000)  # not a multiple of 128: a partial tile
    net = _random_net(gpu, 3, feat, tgt)
    p, norm = net.params()
    got = net.forward(feat)
    want = M.predict(p, norm, feat)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 2e-2 * scale
    assert np.median(np.abs(got - want)) <= 2e-3 * scale
    net.close()


def test_mlp_gradient_matches_oracle(gpu):
    feat, tgt = _data(6, 700)
    net = _random_net(gpu, 4, feat, tgt)
    p, norm = net.params()
    g, loss = net.gradient(feat, tgt)
    l_ref, g_ref = M.loss_grad(p, norm, feat, tgt)
    assert abs(loss - l_ref) <= 1e-3 * l_ref
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        lo = M.OFF[name]
        hi = lo + M.unpack(p)[name].size
        ref = g_ref[lo:hi]
        assert np.linalg.norm(g[lo:hi] - ref) <= 2e-2 * np.linalg.norm(ref) + 1e-7, name
    # and the oracle's rounded gradient is the exact one's up to BF16 effects
    _, g64 = M.loss_grad64(p, norm, feat, tgt)
    assert np.linalg.norm(g - g64) <= 5e-2 * np.linalg.norm(g64)
    net.close()


def test_mlp_training_reduces_loss(gpu):
    feat, tgt = _data(7, 20000)
    net = _random_net(gpu, 5, feat, tgt)
    losses = net.train(feat, tgt, epochs=15, batch=1024, lr=2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.25 * losses[0], losses
    # deterministic: the same seeds give the same weights
    net2 = _random_net(gpu, 5, feat, tgt)
    net2.train(feat, tgt, epochs=2, batch=1024, lr=2e-3, seed=1)
    net3 = _random_net(gpu, 5, feat, tgt)
    net3.train(feat, tgt, epochs=2, batch=1024, lr=2e-3, seed=1)
    assert np.array_equal(net2.params()[0], net3.params()[0])
    for n in (net, net2, net3):
        n.close()


def _mixed(n_worlds=16, n_bodies=48, seed=3):
    from shapes_gb300 import scenes

    return scenes.batched_mixed(seed=seed, n_worlds=n_worlds, n_bodies=n_bodies)


def _batch(gpu, sc):
    return gpu.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], sc["local_xy"])


def _cfg(gpu, sc, iterations=4, learned=False, residual=False):
    c = sc["config"]
    return gpu.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], iterations, learned=learned,
                           residual=residual)


def test_network_off_leaves_the_step_bit_identical(gpu):
    sc = _mixed()
    plain = _batch(gpu, sc)
    plain.step(_cfg(gpu, sc), 60)
    want = plain.get_bodies()
    net = gpu.Mlp(1)
    # attached but the flag is off
    b1 = _batch(gpu, sc)
    b1.set_mlp(net)
    b1.step(_cfg(gpu, sc), 60)
    # flag on but every world's mask cleared
    b2 = _batch(gpu, sc)
    b2.set_mlp(net)
    b2.set_learned_mask(np.zeros(b2.n_worlds, np.uint8))
    b2.step(_cfg(gpu, sc, learned=True), 60)
    assert b2.stats()["predicted"] == 0
    for b in (b1, b2):
        got = b.get_bodies()
        for f in gpu.BODY_FIELDS:
            assert np.array_equal(got[f].view(np.uint64), want[f].view(np.uint64)), f
        b.close()
    plain.close()
    net.close()


def test_predictions_start_the_new_contacts(gpu):
    sc = _mixed()
    warm = 40
    plain = _batch(gpu, sc)
    plain.step(_cfg(gpu, sc), warm)
    plain.step(_cfg(gpu, sc), 1)
    st_plain = plain.stats()
    b = _batch(gpu, sc)
    b.step(_cfg(gpu, sc), warm)
    net = gpu.Mlp(2)
    b.set_mlp(net)
    b.step(_cfg(gpu, sc, learned=True), 1)
    st = b.stats()
    # same poses at the start of the step: the same contacts, and every miss predicted
    assert st["contacts"] == st_plain["contacts"]
    assert st["cache_hits"] == st_plain["cache_hits"]
    assert st["predicted"] == st_plain["contacts"] - st_plain["cache_hits"] > 0
    k_p, lam_p, _ = plain.get_cache()
    k_l, lam_l, _ = b.get_cache()
    assert np.array_equal(k_p, k_l)
    assert not np.array_equal(lam_p, lam_l)  # the new contacts started elsewhere
    b.close()
    plain.close()
    net.close()


def test_sample_collection_matches_the_cache(gpu):
    sc = _mixed()
    b = _batch(gpu, sc)
    b.step(_cfg(gpu, sc), 40)
    b.collect(100000)
    b.step(_cfg(gpu, sc), 1)
    st = b.stats()
    feat, tgt = b.samples()
    assert len(feat) == st["contacts"] - st["cache_hits"] > 0
    assert np.all(np.isfinite(feat)) and np.all(np.isfinite(tgt))
    _, lam, _ = b.get_cache()
    # every target is the final (normal, friction) pair of one of this step's contacts
    have = {(np.float32(a), np.float32(c)) for a, c in lam}
    assert all((a, c) in have for a, c in tgt)
    # pair-count feature is 1 or 2, the static flag 0 or 1
    assert set(np.unique(feat[:, 12])) <= {1.0, 2.0}
    assert set(np.unique(feat[:, 13])) <= {0.0, 1.0}
    b.collect(0)
    b.close()


def test_judge_reverts_worlds_over_the_limit(gpu):
    sc = _mixed()
    b = _batch(gpu, sc)
    b.step(_cfg(gpu, sc), 40)
    net = gpu.Mlp(2)
    b.set_mlp(net)
    zero = np.zeros(b.n_worlds)
    b.set_judge(max_residual=zero)
    b.step(_cfg(gpu, sc, learned=True), 1)
    res, _ = b.world_metrics()
    mask = b.learned_mask()
    # every world with a non-zero residual went back to the plain start
    assert np.array_equal(mask == 0, res > 0)
    assert b.stats()["reverted"] == int((res > 0).sum()) > 0
    # reverted worlds start plainly: only still-masked worlds get predictions
    b.set_judge()
    b.set_learned_mask(np.zeros(b.n_worlds, np.uint8))
    b.step(_cfg(gpu, sc, learned=True), 1)
    assert b.stats()["predicted"] == 0
    b.close()
    net.close()


def test_trained_network_lowers_the_residual_of_new_contacts(gpu):
    """What the network gains: trained on plain runs of one set of mixed
    piles, it starts the new contacts of another set so that, at the same
    sweep count, the solver residual over the impact phase (most contacts
    new) is clearly lower than with the plain zero start."""
    train = _mixed(n_worlds=128, n_bodies=64, seed=11)
    b = _batch(gpu, train)
    b.collect(2_000_000)
    b.step(_cfg(gpu, train, iterations=8), 200)
    feat, tgt = b.samples()
    b.close()
    assert len(feat) > 10000
    net = gpu.Mlp(0)
    net.fit_normalization(feat, tgt)
    losses = net.train(feat, tgt, epochs=20, batch=4096, lr=2e-3, seed=0)
    assert losses[-1] < 0.8 * losses[0]

    test = _mixed(n_worlds=128, n_bodies=64, seed=12)

    def mean_residual(learned, steps=60, iterations=2):
        bb = _batch(gpu, test)
        if learned:
            bb.set_mlp(net)
        tot, pred = 0.0, 0
        for _ in range(steps):
            bb.step(_cfg(gpu, test, iterations=iterations, learned=learned, residual=True), 1)
            pred += bb.stats()["predicted"]
            r = np.empty(bb.n_worlds)
            gpu.check(gpu.lib().shapes_batch_get_world_metrics(bb.handle, r.ctypes.data_as(gpu._dp), None), "m")
            tot += r.mean()
        bb.close()
        return tot / steps, pred

    plain, _ = mean_residual(False)
    learned, predicted = mean_residual(True)
    assert predicted > 0
    assert learned < 0.85 * plain, (learned, plain)
    net.close()


def test_learned_start_on_ragged_and_empty_worlds(gpu):
    """Empty, one-body and static-only worlds next to busy ones: predictions,
    samples and the judge run, empty worlds keep a zero residual and stay
    learned, and two runs give the same bits."""
    from shapes_gb300 import scenes

    sc = scenes.ragged_worlds()
    runs = []
    for _ in range(2):
        b = gpu.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], sc["local_xy"],
                      sc["shape_kind"])
        net = gpu.Mlp(3)
        b.set_mlp(net)
        b.step(_cfg(gpu, sc, learned=True), 20)
        assert b.stats()["predicted"] >= 0
        b.collect(10000)
        b.step(_cfg(gpu, sc, learned=True), 1)
        feat, tgt = b.samples()
        assert np.all(np.isfinite(feat)) and np.all(np.isfinite(tgt))
        b.collect(0)
        b.set_judge(max_residual=np.zeros(b.n_worlds))
        b.step(_cfg(gpu, sc, learned=True), 1)
        res, depth = b.world_metrics()
        assert np.all(np.isfinite(res)) and np.all(np.isfinite(depth))
        assert res[[0, 2, 9]].tolist() == [0.0] * 3
        assert np.array_equal(b.learned_mask() == 0, res > 0)
        runs.append(b.get_bodies())
        b.close()
        net.close()
    for f in gpu.BODY_FIELDS:
        assert np.array_equal(runs[0][f].view(np.uint64), runs[1][f].view(np.uint64)), f
