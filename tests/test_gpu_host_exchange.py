"""cmcg_step_host (upload, step in two graph-replayed halves, read-back that
overlaps the second half) gives exactly what put_stars + step + get_stars
give, with and without graphs, for one cluster and for an uneven ensemble."""
import numpy as np
import pytest

import cmcgpu

pytestmark = pytest.mark.gpu

KEYS = ("r", "m", "vr", "vt", "E", "J", "id")


def _ctx(ics, seed):
    ps = [cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed + i) for i, ic in enumerate(ics)]
    g = cmcgpu.Context([len(ic["r"]) for ic in ics], ps)
    for c, ic in enumerate(ics):
        g.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    return g


def _bufs(n):
    b = {k: np.zeros(n + 8) for k in KEYS[:-1]}
    b["id"] = np.zeros(n + 8, np.int64)
    return b


@pytest.mark.parametrize("sizes", [[20000], [6000, 15000, 9001]])
def test_step_host_equals_put_step_get(gpulib, sizes):
    ics = [cmcgpu.generate(cmcgpu.KING if i % 2 else cmcgpu.PLUMMER, n, seed=90 + i, imf=1)
           for i, n in enumerate(sizes)]
    ref, hx_graph, hx_direct = _ctx(ics, 7), _ctx(ics, 7), _ctx(ics, 7)
    hx_graph.use_graph(True)
    hx_direct.use_graph(False)
    state = {}
    for name, g in (("ref", ref), ("graph", hx_graph), ("direct", hx_direct)):
        bufs = [_bufs(n) for n in sizes]
        ns = [g.get_stars(c, bufs[c]) for c in range(len(sizes))]
        for _ in range(4):
            if name == "ref":
                for c in range(len(sizes)):
                    g.put_stars(c, ns[c], bufs[c])
                g.step(1)
                ns = [g.get_stars(c, bufs[c]) for c in range(len(sizes))]
            else:
                ns = g.step_host([(ns[c], bufs[c]) for c in range(len(sizes))], bufs)
            g.check_device(name)
        state[name] = (ns, bufs)
    for name in ("graph", "direct"):
        ns, bufs = state[name]
        assert ns == state["ref"][0], name
        for c, n in enumerate(ns):
            for k in KEYS:
                assert np.array_equal(bufs[c][k][:n], state["ref"][1][c][k][:n]), (name, c, k)
    for g in (ref, hx_graph, hx_direct):
        g.close()


def test_single_steps_from_part_graphs_equal_direct_steps(gpulib):
    ic = cmcgpu.generate(cmcgpu.KING, 20000, seed=95, imf=1)
    a, b = _ctx([ic], 9), _ctx([ic], 9)
    a.use_graph(True)
    b.use_graph(False)
    for _ in range(3):
        a.step(1)  # four graph launches a step
    a.step(2)      # the two-step graph
    b.step(5)
    for g in (a, b):
        g.check_device("steps")
    for name in ("r", "vr", "vt", "m", "E", "J", "star_phi"):
        assert np.array_equal(a.get(name), b.get(name)), name
    assert np.array_equal(a.ids(), b.ids())


def test_step_host_rejects_short_output(gpulib):
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 5000, seed=97)
    g = _ctx([ic], 11)
    big, small = _bufs(5000), _bufs(100)
    n = g.get_stars(0, big)
    with pytest.raises(cmcgpu.CmcError):
        g.step_host([(n, big)], [small])
    g.close()
