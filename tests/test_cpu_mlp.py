"""CPU checks of the learned proposal's oracle (no GPU).

The GPU tests compare the tensor-core kernels with oracle/mlp.py; these pin
that oracle: its float64 back-propagation against finite differences, its
BF16 mirror against the float64 gradient, the BF16 rounding itself, and the
stored proposal (a monotone CDF whose last bin keeps at least the floor).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp  # noqa: E402


def _records(n, seed):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0.0, 1.0, (n, mlp.NIN)).astype(np.float32)
    bins = rng.integers(0, mlp.NBINS, n)
    ntrial = rng.integers(1, 6, n)
    return feat, bins, ntrial


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -7, -2.5, 3.0e-39], np.float32)
    got = mlp.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0                      # tie: to the even neighbour
    assert got[2] == np.float32(1.0 + 2.0 ** -6)  # tie: to the even neighbour above
    assert got[3] == np.float32(1.0 + 2.0 ** -7)  # representable
    assert got[4] == -2.5
    assert got[5] > 0.0                       # a subnormal float keeps its sign and stays nonzero


def test_exact_gradient_matches_finite_differences():
    w = mlp.init_params(3).astype(np.float64)
    feat, bins, ntrial = _records(48, 4)
    g = mlp.grad_exact(w, feat, bins, ntrial)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(np.arange(lo, hi), 12, replace=False)
                          for lo, hi in [(mlp.P_W1, mlp.P_B1), (mlp.P_B1, mlp.P_W2), (mlp.P_W2, mlp.P_B2),
                                         (mlp.P_B2, mlp.P_W3), (mlp.P_W3, mlp.P_B3), (mlp.P_B3, mlp.NPARAM)]])
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (mlp.loss_exact(wp, feat, bins, ntrial) - mlp.loss_exact(wm, feat, bins, ntrial)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_mirror_close_to_exact_gradient():
    w = mlp.init_params(7)
    feat, bins, ntrial = _records(512, 8)
    gb, (nll, geo) = mlp.grad_bf16(w, feat, bins, ntrial)
    ge = mlp.grad_exact(w, feat, bins, ntrial)
    for lo, hi in [(mlp.P_W1, mlp.P_B1), (mlp.P_B1, mlp.P_W2), (mlp.P_W2, mlp.P_B2), (mlp.P_B2, mlp.P_W3),
                   (mlp.P_W3, mlp.P_B3), (mlp.P_B3, mlp.NPARAM)]:
        err = np.linalg.norm(gb[lo:hi] - ge[lo:hi]) / np.linalg.norm(ge[lo:hi])
        assert err < 0.05, (lo, err)
    nll_e, geo_e = mlp.loss_terms(mlp._forward_exact(w, feat)[0], bins, ntrial)
    assert abs(nll - nll_e.mean()) < 0.02 * nll_e.mean() and abs(geo - geo_e.mean()) < 0.02 * geo_e.mean()


def test_proposal_is_a_monotone_cdf_with_floor():
    rng = np.random.default_rng(9)
    z = rng.normal(0.0, 8.0, (200, mlp.NOUT))
    out = mlp.proposal(z)
    cdf = out[:, :mlp.NBINS - 1]
    step = np.diff(np.concatenate([np.zeros((200, 1)), cdf, np.ones((200, 1))], axis=1), axis=1)
    assert np.all(step >= mlp.FLOOR / mlp.NBINS * (1 - 1e-12))
    assert np.allclose(step.sum(axis=1), 1.0)
    assert np.all((out[:, -1] > 0) & (out[:, -1] < 1))


def test_adam_step_moves_each_parameter_by_lr_first():
    w = mlp.init_params(2)
    g = np.random.default_rng(1).normal(size=w.size).astype(np.float32)
    w1, m, v = mlp.adam_step(w, np.zeros_like(w), np.zeros_like(w), g, 1, 1e-3)
    assert np.allclose(np.abs(w1 - w), 1e-3, rtol=1e-3)
    assert np.all(np.sign(w - w1) == np.sign(g))
