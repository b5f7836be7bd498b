"""The learned starting point of the GRMHD Newton cons2prim on the device.

* The tensor-core training kernels' gradient and the inference kernel's
  outputs against the oracle's FP64 restatement (oracle/mlp_ref.py) with the
  same BF16 roundings of the operands.
* Training on pairs harvested from the Kerr torus's own cons2prim solves
  (features including the previous primitives; targets the change of
  log(W^2 - 1) and log(P / rho) to the converged solution) reduces the loss.
* With the trained network attached, the Newton iteration converges to the
  same primitives (relative L1 1e-13 per component after the steps) and the
  mean iteration at first convergence (k_converge) is reported against the
  reference's own start, the previous primitives."""
import numpy as np
import pytest

from oracle import mlp_ref
from test_gpu_parity import _domain

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


F = 10   # features


def _random_norm(rng):
    return np.concatenate([rng.normal(0, 1, F), rng.uniform(0.5, 2, F), rng.normal(0, 1, 2),
                           rng.uniform(0.5, 2, 2)]).astype(np.float32)


def test_mlp_gradient_matches_restatement():
    import disco_gb300 as dg
    rng = np.random.default_rng(5)
    m = dg.Mlp(seed=11, capacity=16)
    p, _ = m.params()
    norm = _random_norm(rng)
    m.set_params(norm=norm)
    n = 333                                      # not a multiple of the 16-sample tile
    X = (rng.normal(0, 1.5, (n, F)) * norm[F:2 * F] + norm[:F]).astype(np.float32)
    Y = (rng.normal(0, 1.5, (n, 2)) * norm[2 * F + 2:] + norm[2 * F:2 * F + 2]).astype(np.float32)
    loss, g = m.grad(X, Y)
    l_ref, g_ref, _ = mlp_ref.forward_backward(p, norm, X, Y, bf16=True)
    assert loss == pytest.approx(l_ref, rel=1e-3)
    gd, gr = mlp_ref.unpack(g), mlp_ref.unpack(g_ref)
    errs = {k: _rel_l2(gd[k], gr[k]) for k in gr}
    print("relative L2 error of the device gradient per parameter block:", errs)
    for k, e in errs.items():
        assert e < 1e-2, (k, e)
    # and against the plain FP64 network: the BF16 operands cost little
    _, g64, _ = mlp_ref.forward_backward(p, norm, X, Y, bf16=False)
    assert _rel_l2(g, g64) < 5e-2
    m.close()


def test_mlp_inference_matches_restatement():
    import disco_gb300 as dg
    rng = np.random.default_rng(6)
    m = dg.Mlp(seed=12, capacity=16)
    p, _ = m.params()
    norm = _random_norm(rng)
    m.set_params(norm=norm)
    X = (rng.normal(0, 1.5, (1000, F)) * norm[F:2 * F] + norm[:F]).astype(np.float32)
    Yd = m.predict(X)
    _, _, Yr = mlp_ref.forward_backward(p, norm, X, np.zeros((1000, 2)), bf16=True)
    for o in range(2):   # in standardised units
        yd = (Yd[:, o] - norm[2 * F + o]) / norm[2 * F + 2 + o]
        yr = (Yr[:, o] - norm[2 * F + o]) / norm[2 * F + 2 + o]
        assert np.max(np.abs(yd - yr)) <= 2e-3 * max(1.0, np.abs(yr).max()), o
    m.close()


def _harvest_and_train(m, steps=12, train_steps=3000):
    d, _ = _domain("cfg4t_n24", 0)
    m.harvest(d, stride=1, steps=steps)
    d.close()
    m.fit_norm()
    return m.train(train_steps, batch=4096, lr=2e-3, seed=3)


def test_training_reduces_loss_and_guess_keeps_the_solution():
    """Trains on harvested solves, then advances the same torus from the same
    start with the reference's start (plain) and with the learned one under
    a few gates (the learned start is taken where its residual is below a
    ratio times that of the previous primitives).  The solution must not
    change.  The mean k_converge of each is printed; on this torus the
    previous primitives are already a close start (mean k_converge about
    2.6) and the learned start does not lower it, so the bar is only that
    the best gate costs at most 5 % more."""
    import disco_gb300 as dg
    m = dg.Mlp(seed=13, capacity=1 << 20)
    l0, l1 = _harvest_and_train(m)
    print("loss: first batch", l0, "last batch", l1)
    assert l1 < 0.1 * l0
    a, g = _domain("cfg4t_n24", 0)
    floors = (1.0, 0.1, 1e-2, 1e-3, 1e-4)   # gate ratios
    bs = []
    for f in floors:
        b, _ = _domain("cfg4t_n24", 0)
        m.set_gate(0.0, f)
        b.attach_guess(m)
        b.c2p_stats(reset=True)
        bs.append(b)
    a.c2p_stats(reset=True)
    for _ in range(3):
        dt = a.getmindt()
        a.timestep(dt)
        for b in bs:
            b.timestep(dt)
    sa = a.c2p_stats()
    ka = sa["kconv"] / sa["calls"]
    pa = a.state()["prim"]
    real = g["real"].astype(bool)
    kbs = []
    for f, b in zip(floors, bs):
        sb = b.c2p_stats()
        assert sa["calls"] == sb["calls"] > 0
        kb = sb["kconv"] / sb["calls"]
        kbs.append(kb)
        print(f"gate ratio {f:g}: mean k_converge plain {ka:.3f}, learned {kb:.3f}, ratio {ka / kb:.3f}; "
              f"guess used in {sb['guessed'] / sb['calls']:.4f} of the calls")
        pb = b.state()["prim"]
        for q in range(pa.shape[0]):
            den = np.abs(pa[q, real]).sum()
            if den > 0:
                assert np.abs(pb[q, real] - pa[q, real]).sum() <= 1e-13 * den, (f, q)
        # a learned start may converge where the previous primitives stop at
        # the iteration cap (the atmosphere at the density floor), never the
        # other way round: a start that does not converge falls back
        assert b.status()["c2p_no_converge"] <= a.status()["c2p_no_converge"]
    assert bs[0].c2p_stats()["guessed"] > 0
    assert min(kbs) <= 1.05 * ka
    a.close(); m.close()
    for b in bs:
        b.close()
