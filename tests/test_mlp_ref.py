"""The oracle's FP64 restatement of the cons2prim MLP (oracle/mlp_ref.py)
pinned on the CPU: its gradient equals centred finite differences of its
own loss (plain FP64, no BF16 rounding), and its BF16 rounding is
round-to-nearest-even.  The device's tensor-core gradients are checked
against this restatement in tests/test_gpu_mlp.py."""
import numpy as np

from oracle import mlp_ref


def _random_model(rng):
    p = np.zeros(mlp_ref.NPARAMS)
    w = mlp_ref.unpack(p)
    w["W1"][:, :10] = rng.normal(0, 0.4, (64, 10))
    w["W2"][...] = rng.normal(0, 0.2, (64, 64))
    w["W3"][:2] = rng.normal(0, 0.2, (2, 64))
    w["b1"][...] = rng.normal(0, 0.1, 64)
    w["b2"][...] = rng.normal(0, 0.1, 64)
    w["b3"][:2] = rng.normal(0, 0.1, 2)
    norm = np.concatenate([rng.normal(0, 1, 10), rng.uniform(0.5, 2, 10), rng.normal(0, 1, 2),
                           rng.uniform(0.5, 2, 2)])
    return mlp_ref.pack(w), norm


def test_fp64_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p, norm = _random_model(rng)
    X = rng.normal(0, 1.5, (37, 10))
    Y = rng.normal(0, 1.5, (37, 2))
    _, g, _ = mlp_ref.forward_backward(p, norm, X, Y, bf16=False)
    live = np.flatnonzero(g)
    idx = rng.choice(live, 200, replace=False)
    n = len(X)
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = mlp_ref.forward_backward(pp, norm, X, Y, bf16=False)[0] / n
        lm = mlp_ref.forward_backward(pm, norm, X, Y, bf16=False)[0] / n
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    # the padded parameters (inputs 10..15 of W1, rows 2..7 of W3) get no gradient
    w = mlp_ref.unpack(g)
    assert not np.any(w["W1"][:, 10:]) and not np.any(w["W3"][2:]) and not np.any(w["b3"][2:])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.001953125, 1.0029296875, -3.1415926, 65504.0, 1e-40])
    r = mlp_ref.to_bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                          # 1 + 2^-8 is a tie: to the even neighbour 1.0
    assert r[3] == 1.0                          # below the tie
    assert r[2] == 1.0078125                    # above the tie
    assert abs(r[5] + 3.140625) < 1e-12
    # every value is representable in 8 bits of significand
    m, e = np.frexp(r[np.isfinite(r) & (r != 0)])
    assert np.all(np.abs(m * 256 - np.round(m * 256)) == 0)
