"""CPU checks of the network's oracle (oracle/mlp_oracle.py): BF16 rounding,
back-propagation against central finite differences, and the BF16-rounded
gradient against the unrounded one."""
import numpy as np

from oracle import mlp_oracle as M


def _net(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAMS, dtype=np.float32)
    for k, (fo, fi) in {"W1": (64, 16), "W2": (64, 64), "W3": (64, 64), "W4": (2, 64)}.items():
        p[M.OFF[k]:M.OFF[k] + fo * fi] = rng.uniform(-1, 1, fo * fi) * np.sqrt(6.0 / fi)
    for k in ("b1", "b2", "b3"):
        p[M.OFF[k]:M.OFF[k] + 64] = rng.normal(0, 0.1, 64)
    p[M.OFF["b4"]:] = rng.normal(0, 0.1, 2)
    norm = M.identity_norm()
    norm[:16] = rng.normal(0, 0.5, 16)
    norm[16:32] = rng.uniform(0.5, 2.0, 16)
    norm[32:34] = rng.normal(0, 1, 2)
    norm[34:36] = rng.uniform(0.5, 2.0, 2)
    return p, norm.astype(np.float32), rng


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0, 65536.0 + 256.0],
                 dtype=np.float32)
    got = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties to even gives 1.0;
    # 1 + 3 * 2^-9 is above the tie and rounds up to 1 + 2^-7
    want = np.array([1.0, 1.0, 1.0, 1.0 + 2 ** -7, -2.5, 0.0, 65536.0], dtype=np.float32)
    assert np.array_equal(got, want), (got, want)
    assert np.isnan(M.bf16(np.float32(np.nan)))


def test_backprop_matches_finite_differences():
    p, norm, rng = _net(1)
    feat = rng.normal(0, 1.5, (24, 16)).astype(np.float32)
    tgt = rng.normal(0, 1.0, (24, 2)).astype(np.float32)
    loss, g = M.loss_grad64(p, norm, feat, tgt)
    idx = rng.choice(M.N_PARAMS, 80, replace=False)
    p64 = p.astype(np.float64)
    for k in idx:
        e = 1e-6
        a, b = p64.copy(), p64.copy()
        a[k] += e
        b[k] -= e
        fd = (M.loss_grad64(a, norm, feat, tgt)[0] - M.loss_grad64(b, norm, feat, tgt)[0]) / (2 * e)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(g[k]), (k, fd, g[k])


def test_rounded_gradient_close_to_exact():
    p, norm, rng = _net(2)
    feat = rng.normal(0, 1.5, (512, 16)).astype(np.float32)
    tgt = rng.normal(0, 1.0, (512, 2)).astype(np.float32)
    l1, g1 = M.loss_grad(p, norm, feat, tgt)
    l2, g2 = M.loss_grad64(p, norm, feat, tgt)
    assert abs(l1 - l2) <= 2e-2 * l2
    assert np.linalg.norm(g1 - g2) <= 3e-2 * np.linalg.norm(g2)
