"""Batched ensembles: many clusters of uneven N in one context (one launch per
kernel, segmented sort and scans, one CUDA graph for the whole step).  Each
cluster must evolve exactly as it does alone."""
import numpy as np
import pytest

import cmcgpu

pytestmark = pytest.mark.gpu


def _ensemble_spec(n, master=2026, lo=2000, hi=40000):
    """Alternating Plummer / King (W0 in {3,5,7,9}) with Kroupa masses and N
    log-uniform in [lo, hi]; per-cluster seeds derived from one master seed
    (the shape of the 128-cluster benchmark ensemble, scaled down)."""
    rng = np.random.default_rng(master)
    Ns = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(int)
    out = []
    for i, N in enumerate(Ns):
        seed = cmcgpu.derive_seed(master, i)
        if i % 2 == 0:
            ic = cmcgpu.generate(cmcgpu.PLUMMER, int(N), seed=seed, imf=1)
        else:
            ic = cmcgpu.generate(cmcgpu.KING, int(N), seed=seed, w0=float(rng.choice([3, 5, 7, 9])), imf=1)
        out.append((int(N), ic, seed))
    return out


def _state(ctx, c):
    s = {k: ctx.get(k, c) for k in ("r", "m", "vr", "vt", "E", "J", "star_phi")}
    s["ids"] = ctx.ids(c)
    for k in ("Etot", "Mtotal", "Rtidal", "Dt", "max_r"):
        s[k] = ctx.scalar(k, c)
    return s


@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_clusters_evolve_as_they_do_alone(gpulib, graph):
    spec = _ensemble_spec(9)
    params = [gpulib.default_params(orbit_r=ic["rtid"], seed=seed) for N, ic, seed in spec]
    ens = gpulib.Context([N for N, _, _ in spec], params)
    for c, (N, ic, seed) in enumerate(spec):
        ens.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    ens.initialize()
    if graph:
        ens.use_graph(True)
    ens.step(4)
    ens.check_device("ensemble")
    for c, (N, ic, seed) in enumerate(spec):
        one = gpulib.Context([N], params[c])
        one.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        one.initialize()
        one.step(4)
        one.check_device("single")
        a, b = _state(ens, c), _state(one, 0)
        for k in a:
            assert np.array_equal(a[k], b[k]), (c, k)
        one.close()
    ens.close()
