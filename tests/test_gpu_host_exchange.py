"""cmcg_step_host (upload, step in graph-replayed parts, copies that overlap
them) gives exactly what put_stars + step + get_stars give, with and without
graphs, for one cluster and for an uneven ensemble.  The caller's E and J
arrive during the relaxation and are merged in for the stars it leaves alone:
with the relaxation off that is every star."""
import numpy as np
import pytest

import cmcgpu

pytestmark = pytest.mark.gpu

KEYS = ("r", "m", "vr", "vt", "E", "J", "id")


def _ctx(ics, seed, **kw):
    ps = [cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed + i, **kw) for i, ic in enumerate(ics)]
    g = cmcgpu.Context([len(ic["r"]) for ic in ics], ps)
    for c, ic in enumerate(ics):
        g.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    return g


def _bufs(n, pinned=False):
    """Host star arrays: pageable numpy arrays, or views of pinned (page-locked)
    memory, which the batched exchange reads and writes from the device."""
    if pinned:
        import torch

        b = {k: torch.zeros(n + 8, dtype=torch.float64, pin_memory=True).numpy() for k in KEYS[:-1]}
        b["id"] = torch.zeros(n + 8, dtype=torch.int64, pin_memory=True).numpy()
        return b
    b = {k: np.zeros(n + 8) for k in KEYS[:-1]}
    b["id"] = np.zeros(n + 8, np.int64)
    return b


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
@pytest.mark.parametrize("sizes", [[20000], [6000, 15000, 9001]])
def test_step_host_equals_put_step_get(gpulib, sizes, pinned):
    """Pinned arrays go through the batched exchange (the exposed uploads and
    the E, J downloads by one kernel launch each, over every cluster),
    pageable ones through the copy engines, one copy per array; both must
    give put_stars + step + get_stars.  "inplace" steps a HostStars binding
    (the same cmcg_stars array as input and output)."""
    ics = [cmcgpu.generate(cmcgpu.KING if i % 2 else cmcgpu.PLUMMER, n, seed=90 + i, imf=1)
           for i, n in enumerate(sizes)]
    ref, hx_graph, hx_direct, hx_inplace = _ctx(ics, 7), _ctx(ics, 7), _ctx(ics, 7), _ctx(ics, 7)
    hx_graph.use_graph(True)
    hx_direct.use_graph(False)
    hx_inplace.use_graph(True)
    state = {}
    for name, g in (("ref", ref), ("graph", hx_graph), ("direct", hx_direct), ("inplace", hx_inplace)):
        bufs = [_bufs(n, pinned and name != "ref") for n in sizes]
        ns = [g.get_stars(c, bufs[c]) for c in range(len(sizes))]
        hs = cmcgpu.HostStars(bufs, ns) if name == "inplace" else None
        for _ in range(4):
            if name == "ref":
                for c in range(len(sizes)):
                    g.put_stars(c, ns[c], bufs[c])
                g.step(1)
                ns = [g.get_stars(c, bufs[c]) for c in range(len(sizes))]
            elif hs is not None:
                ns = g.step_host_inplace(hs)
            else:
                ns = g.step_host([(ns[c], bufs[c]) for c in range(len(sizes))], bufs)
            g.check_device(name)
        state[name] = (ns, bufs)
    for name in ("graph", "direct", "inplace"):
        ns, bufs = state[name]
        assert ns == state["ref"][0], name
        for c, n in enumerate(ns):
            for k in KEYS:
                assert np.array_equal(bufs[c][k][:n], state["ref"][1][c][k][:n]), (name, c, k)
    for g in (ref, hx_graph, hx_direct, hx_inplace):
        g.close()


@pytest.mark.parametrize("relaxation,fp32", [(0, 0), (1, 0), (1, 1)])
def test_step_host_takes_callers_E_J(gpulib, relaxation, fp32):
    # E and J changed on the host between steps: without relaxation the
    # orbits read them for every star, with it (FP64 or FP32 kinematics) for
    # the unpaired last star
    ic = cmcgpu.generate(cmcgpu.KING, 12001, seed=98, imf=1)
    out = {}
    for name in ("ref", "graph", "direct"):
        g = _ctx([ic], 13, RELAXATION=relaxation, relax_fp32=fp32)
        g.use_graph(name == "graph")
        b = _bufs(12001)
        n = g.get_stars(0, b)
        for _ in range(3):
            b["E"][:n] *= 1.0 + 1e-7
            b["J"][:n] *= 1.0 - 1e-7
            if name == "ref":
                g.put_stars(0, n, b)
                g.step(1)
                n = g.get_stars(0, b)
            else:
                (n,) = g.step_host([(n, b)], [b])
            g.check_device(name)
        out[name] = (n, b)
        g.close()
    for name in ("graph", "direct"):
        assert out[name][0] == out["ref"][0], name
        n = out[name][0]
        for k in KEYS:
            assert np.array_equal(out[name][1][k][:n], out["ref"][1][k][:n]), (name, k)


def test_step_host_with_learned_proposal(gpulib):
    # the learned sampler's passes read E and J after the merge like the plain one
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 20000, seed=99, imf=0)
    out = {}
    for name in ("ref", "hx"):
        g = _ctx([ic], 15)
        g.mlp_init(3)
        g.set_learned(cmcgpu.LEARN_ON, 1.2)
        g.use_graph(name == "hx")
        b = _bufs(20000)
        n = g.get_stars(0, b)
        for _ in range(3):
            if name == "ref":
                g.put_stars(0, n, b)
                g.step(1)
                n = g.get_stars(0, b)
            else:
                (n,) = g.step_host([(n, b)], [b])
            g.check_device(name)
        out[name] = (n, b)
        g.close()
    assert out["hx"][0] == out["ref"][0]
    n = out["hx"][0]
    for k in KEYS:
        assert np.array_equal(out["hx"][1][k][:n], out["ref"][1][k][:n]), k


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


def test_step_host_on_device_arrays(gpulib):
    """The caller's arrays in device memory: the kernels reach them like pinned
    host arrays and the copies take their direction from unified addressing.
    Three steps in place give what they give on pinned host arrays."""
    import torch

    ic = cmcgpu.generate(cmcgpu.KING, 20000, seed=95, imf=1)
    a, b = _ctx([ic], 7), _ctx([ic], 7)
    a.use_graph(True)
    b.use_graph(True)
    bufs = _bufs(20000, pinned=True)
    n = a.get_stars(0, bufs)
    dev = {k: torch.from_numpy(bufs[k].copy()).cuda() for k in KEYS}
    torch.cuda.synchronize()
    hs = cmcgpu.HostStars([bufs], [n])
    arr = (cmcgpu.Stars * 1)()
    arr[0] = cmcgpu.Stars(n, len(bufs["r"]), *[dev[k].data_ptr() for k in KEYS])
    for _ in range(3):
        a.step_host_inplace(hs)
        assert cmcgpu.lib().cmcg_step_host(b._h, arr, arr) == 0
        b.check_device("device arrays")
    (n1,) = hs.counts()
    assert arr[0].N == n1
    for k in KEYS:
        assert np.array_equal(dev[k][:n1].cpu().numpy(), bufs[k][:n1]), k
    a.close()
    b.close()
