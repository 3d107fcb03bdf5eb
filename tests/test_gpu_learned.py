"""The learned proposal on the GPU: tensor-core network against the CPU
oracle (oracle/mlp.py), the sampler's exactness guarantees, and what the
trained network gains over the plain sampler.

* forward logits and stored proposal, gradient (a training pass) and the
  Adam step against the oracle's BF16 mirror;
* the learned launch sequence with plain trials only (collect mode), and the
  proposal with an envelope too small to hold anywhere (every star goes back
  to the plain sampler), both give the plain sampler's results bit for bit;
* trained on records the plain sampler produced, the proposal needs fewer
  trials per star, and the radii it samples follow the plain sampler's
  distribution (two-sample Kolmogorov-Smirnov test on X).
"""
import numpy as np
import pytest

import cmcgpu
import mlp

pytestmark = pytest.mark.gpu


def _records(n, seed):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0.0, 1.0, (n, mlp.NIN)).astype(np.float32)
    bins = rng.integers(0, mlp.NBINS, n).astype(np.int32)
    ntrial = rng.integers(1, 6, n).astype(np.int32)
    return feat, bins, ntrial


@pytest.fixture(scope="module")
def net_ctx(gpulib):
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 2000, seed=3)
    g = cmcgpu.Context([2000], cmcgpu.default_params(orbit_r=ic["rtid"], seed=5))
    yield g
    g.close()


def _blocks():
    return [("W1", mlp.P_W1, mlp.P_B1), ("b1", mlp.P_B1, mlp.P_W2), ("W2", mlp.P_W2, mlp.P_B2),
            ("b2", mlp.P_B2, mlp.P_W3), ("W3", mlp.P_W3, mlp.P_B3), ("b3", mlp.P_B3, mlp.NPARAM)]


@pytest.mark.parametrize("n", [1, 127, 1000, 20000])
def test_forward_matches_oracle(net_ctx, n):
    w = mlp.init_params(11)
    net_ctx.mlp_set_params(w)
    assert np.array_equal(net_ctx.mlp_params(), w)
    feat, _, _ = _records(n, 12)
    z, prop = net_ctx.mlp_forward(feat)
    zo, _ = mlp.forward(w, feat)
    err = np.abs(z - zo) / np.maximum(1.0, np.abs(zo))
    # FP32 tensor-core sums against float64 ones; a BF16 activation whose
    # rounding those differences flip moves a logit by ~1e-3 at most
    assert np.median(err) < 1e-5 and err.max() < 1e-2, (np.median(err), err.max())
    # the stored proposal is the oracle's from the kernel's own logits
    po = mlp.proposal(z)
    assert np.abs(prop - po).max() < 2e-6
    assert np.all(np.diff(prop[:, :31], axis=1) > 0) and np.all(prop[:, 30] < 1.0)


@pytest.mark.parametrize("n", [128, 1000, 50000])
def test_gradient_matches_oracle(net_ctx, n):
    w = mlp.init_params(21)
    net_ctx.mlp_set_params(w)
    feat, bins, ntrial = _records(n, 22)
    g, (nll, geo) = net_ctx.mlp_gradient(feat, bins, ntrial)
    go, (nllo, geoo) = mlp.grad_bf16(w, feat, bins, ntrial)
    for name, lo, hi in _blocks():
        err = np.linalg.norm(g[lo:hi] - go[lo:hi]) / np.linalg.norm(go[lo:hi])
        assert err < 1e-2, (name, err)
    assert abs(nll - nllo) <= 1e-4 * nllo and abs(geo - geoo) <= 1e-4 * geoo
    # and the BF16 mirror is the float64 gradient within BF16's resolution
    ge = mlp.grad_exact(w, feat, bins, ntrial)
    assert np.linalg.norm(g - ge) / np.linalg.norm(ge) < 0.05


def test_adam_step_matches_oracle(net_ctx):
    w = mlp.init_params(31)
    net_ctx.mlp_set_params(w)
    feat, bins, ntrial = _records(3000, 32)
    batch, lr, seed = 1024, 1e-3, 77
    loss = net_ctx.mlp_train(feat, bins, ntrial, steps=1, batch=batch, lr=lr, seed=seed)
    idx = mlp.sample_index(seed, 0, np.arange(batch), len(feat))
    go, (nll, geo) = mlp.grad_bf16(w, feat[idx], bins[idx], ntrial[idx])
    wo, _, _ = mlp.adam_step(w, np.zeros_like(w), np.zeros_like(w), go, 1, lr)
    wg = net_ctx.mlp_params()
    # the first Adam step moves each parameter by lr in the gradient's sign;
    # only gradients within rounding of zero may differ in sign
    off = np.abs(wg - wo) > 0.1 * lr
    assert off.mean() < 0.01, off.mean()
    assert abs(loss[0, 0] - nll) <= 1e-4 * nll and abs(loss[0, 1] - geo) <= 1e-4 * geo


def _pair(model, N, seed, w0=6.0, imf=0):
    ic = cmcgpu.generate(model, N, seed=seed, w0=w0, imf=imf)
    out = []
    for _ in range(2):
        g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed + 1))
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        out.append(g)
    return out


def _same_state(a, b):
    for name in ("r", "vr", "vt", "m", "E", "J", "star_phi"):
        assert np.array_equal(a.get(name), b.get(name)), name
    assert np.array_equal(a.ids(), b.ids())


def test_collect_mode_is_the_plain_sampler(gpulib):
    a, b = _pair(cmcgpu.KING, 20000, 41, imf=1)
    b.set_learned(cmcgpu.LEARN_COLLECT)
    for _ in range(3):
        a.step(1)
        b.step(1)
        a.check_device("plain")
        b.check_device("collect")
        feat, X, nt = b.learned_samples()
        assert len(X) > 0.9 * b.nstars() and np.all(nt > 0)
        assert np.all((X >= 0) & (X < 1)) and np.all(np.isfinite(feat))
    _same_state(a, b)
    st = b.learned_stats()
    assert st["stars"] == 0 and st["plain_stars"] > 0.9 * b.nstars()


def test_envelope_that_never_holds_gives_the_plain_sampler(gpulib):
    a, b = _pair(cmcgpu.PLUMMER, 20000, 43)
    b.mlp_init(5)
    b.set_learned(cmcgpu.LEARN_ON, kappa=1e-30)
    for _ in range(2):
        a.step(1)
        b.step(1)
        a.check_device("plain")
        b.check_device("learned")
        st = b.learned_stats()
        assert st["stars"] > 0 and st["failed"] == st["stars"] and st["accepted"] == 0
    _same_state(a, b)


@pytest.fixture(scope="module")
def trained(gpulib):
    """A network trained on a Plummer model's plain-sampler records."""
    N = 100000
    ic = cmcgpu.generate(cmcgpu.PLUMMER, N, seed=51)
    g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=52))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    g.set_learned(cmcgpu.LEARN_COLLECT)
    feats, Xs, nts = [], [], []
    for _ in range(8):
        g.step(1)
        g.check_device("collect")
        f, X, nt = g.learned_samples()
        feats.append(f)
        Xs.append(X)
        nts.append(nt)
    feat, X, nt = np.concatenate(feats), np.concatenate(Xs), np.concatenate(nts)
    bins = np.minimum((X * 32).astype(np.int32), 31)
    g.mlp_init(7)
    loss = g.mlp_train(feat, bins, nt, steps=600, batch=8192, lr=2e-3, seed=9)
    w = g.mlp_params()
    g.close()
    # what a proposal without the network reaches on the same records: the
    # marginal bin frequencies for every star, and one P for every star
    h = np.bincount(bins, minlength=mlp.NBINS) / len(bins)
    nll0 = float(-(h[h > 0] * np.log(h[h > 0])).sum())
    P0 = 1.0 / nt.mean()
    geo0 = float(np.mean((nt - 1) * -np.log(1 - P0) - np.log(P0)))
    return {"w": w, "loss": loss, "plain_trials": float(nt.mean()), "n": len(X), "base": (nll0, geo0)}


def test_training_beats_the_network_free_proposal(trained):
    loss = trained["loss"]
    assert np.all(np.isfinite(loss))
    nll0, geo0 = trained["base"]
    last = loss[-50:].mean(axis=0)
    assert last.sum() < nll0 + geo0 - 0.01, (last, trained["base"])


def test_learned_proposal_samples_the_plain_distribution(trained):
    from scipy.stats import ks_2samp

    a, b = _pair(cmcgpu.PLUMMER, 100000, 61)
    b.mlp_set_params(trained["w"])
    b.set_learned(cmcgpu.LEARN_ON, kappa=1.2)
    a.set_learned(cmcgpu.LEARN_COLLECT)  # the plain sampler, with its records
    a.step(1)
    b.step(1)
    a.check_device("plain")
    b.check_device("learned")
    _, Xa, nta = a.learned_samples()
    _, Xb, ntb = b.learned_samples()
    st = b.learned_stats()
    # fewer trials per star than the plain sampler (the gain of the network)
    learned_trials = (st["trials"] + st["plain_trials"]) / (st["accepted"] + st["plain_stars"])
    plain_trials = float(nta.mean())
    # (about kappa trials when the network has learned the density and P)
    assert learned_trials < 0.75 * plain_trials, (learned_trials, plain_trials, st)
    assert st["failed"] < 0.01 * st["stars"], st
    # the same distribution of the sampling variable (the stars sent back to
    # the plain sampler share its draws, which only makes the test milder)
    p = ks_2samp(Xa, Xb).pvalue
    assert p > 0.01, (p, st)


@pytest.mark.parametrize("model,N,imf", [(cmcgpu.PLUMMER, 50000, 0), (cmcgpu.KING, 50000, 1)])
def test_learned_filter_decisions_match_exact(trained, model, N, imf):
    """Every certified FP32 decision of a proposal trial (accept, or reject,
    with the envelope certainly holding) is re-evaluated exactly
    (check_filters); a disagreement is CMCG_ERR_FILTER."""
    ic = cmcgpu.generate(model, N, seed=71, imf=imf)
    g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=72, check_filters=1))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    g.mlp_set_params(trained["w"])
    for kappa in (1.05, 1.2, 2.0):
        g.set_learned(cmcgpu.LEARN_ON, kappa=kappa)
        g.step(1)
        g.check_device(f"learned step, kappa {kappa}")
        st = g.learned_stats()
        assert st["accepted"] > 0.5 * st["stars"], st  # tight envelopes send more stars back
    g.close()


def test_ensemble_collect_and_tiny_envelope_are_the_plain_sampler(gpulib):
    """Three clusters of uneven N in one context: the learned launch sequence
    with plain trials, and the proposal with an envelope that never holds,
    both reproduce the plain step bit for bit in every cluster."""
    sizes = [7000, 16001, 11000]
    ics = [cmcgpu.generate(cmcgpu.KING if i % 2 else cmcgpu.PLUMMER, n, seed=100 + i, imf=1)
           for i, n in enumerate(sizes)]

    def make():
        ps = [cmcgpu.default_params(orbit_r=ic["rtid"], seed=200 + i) for i, ic in enumerate(ics)]
        g = cmcgpu.Context(sizes, ps)
        for c, ic in enumerate(ics):
            g.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        return g

    plain, collect, tiny = make(), make(), make()
    collect.set_learned(cmcgpu.LEARN_COLLECT)
    tiny.mlp_init(9)
    tiny.set_learned(cmcgpu.LEARN_ON, kappa=1e-30)
    for g in (plain, collect, tiny):
        g.step(2)
        g.check_device("ensemble steps")
    for g in (collect, tiny):
        for c in range(len(sizes)):
            for name in ("r", "vr", "vt", "E", "J", "X"):
                assert np.array_equal(g.get(name, c), plain.get(name, c)), (c, name)
            assert np.array_equal(g.ids(c), plain.ids(c))
    for c in range(len(sizes)):
        _, X, nt = collect.learned_samples(c)
        assert len(X) > 0.9 * collect.nstars(c) and np.all(nt > 0)
    for g in (plain, collect, tiny):
        g.close()


def test_fifty_steps_with_the_proposal_follow_the_plain_run(trained):
    """Config 4's comparison: 50 steps with the proposal and 50 with the plain
    sampler from the same model.  The runs draw differently, so they are two
    realisations: their energy errors stay at the plain run's level and their
    Lagrange radii agree to the noise of 1e5 stars."""
    N = 100000
    ic = cmcgpu.generate(cmcgpu.PLUMMER, N, seed=111)
    runs = {}
    for mode in (cmcgpu.LEARN_OFF, cmcgpu.LEARN_ON):
        g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=112))
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        g.mlp_set_params(trained["w"])
        g.set_learned(mode, kappa=1.2)
        e0 = g.scalar("Etot")
        g.use_graph(True)
        g.step(50)
        g.check_device(f"50 steps, mode {mode}")
        d = g.diagnostics(mass_pc=[0.1, 0.5, 0.9])
        runs[mode] = (abs(g.scalar("Etot") - e0) / abs(e0) / 50, d.arr("mass_r"), g.nstars(), d.rh)
        g.close()
    (ep, lp, np_, rhp), (el, ll, nl, rhl) = runs[cmcgpu.LEARN_OFF], runs[cmcgpu.LEARN_ON]
    print(f"plain: dE/E/step {ep:.2e}, Lagrange radii {lp}, rh {rhp:.5f}, N {np_}; "
          f"learned: {el:.2e}, {ll}, {rhl:.5f}, {nl}")
    assert ep < 1e-6 and el < 1e-6, (ep, el)
    assert np.all(np.abs(ll / lp - 1) < 0.02), (lp, ll)
    assert abs(rhl / rhp - 1) < 0.02 and abs(nl - np_) <= 0.001 * N, (rhp, rhl, np_, nl)
