"""The allocation-free radius sort (cmcg_sort_radii_noalloc) against the
context's own sort (cmcg_qsorts_new), through the C ABI.

Callers that cannot allocate device memory while running use this entry point;
it must order the stars exactly as the regular sort does.  Two calls in a row
with different inputs check that the shared fixed scratch array carries no
state from one call into the next.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _context_order(gpulib, radii):
    """Permutation produced by the regular sort of a context."""
    n = len(radii)
    ic = gpulib.generate(gpulib.PLUMMER, n, seed=3)
    ctx = gpulib.Context([n], gpulib.default_params(orbit_r=ic["rtid"]))
    ctx.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], np.arange(1, n + 1))
    ctx.set("rnew", radii)
    ctx.qsorts_new()
    ctx.check_device("qsorts_new")
    order = ctx.ids() - 1  # ids were 1..n in input order
    ctx.close()
    return order


def _noalloc_order(gpulib, radii):
    import torch

    d_r = torch.tensor(radii, dtype=torch.float64, device="cuda:0")
    d_perm = torch.empty(len(radii), dtype=torch.int32, device="cuda:0")
    nb = C.c_long(-1)
    rc = gpulib.lib().cmcg_sort_radii_noalloc(C.c_void_p(d_r.data_ptr()), len(radii), C.c_void_p(d_perm.data_ptr()),
                                             C.byref(nb), None)
    assert rc == 0
    torch.cuda.synchronize()
    return d_perm.cpu().numpy().astype(np.int64), nb.value


def test_noalloc_sort_matches_regular_sort_twice(gpulib):
    rng = np.random.default_rng(2024)
    for n in (70001, 12345):  # two calls in a row on the shared scratch array
        radii = np.exp(rng.uniform(-6.0, 5.0, size=n))
        radii[rng.random(n) < 0.01] = 1e10  # escapers go last and are dropped
        radii[5] = radii[7]  # a tie keeps input order
        want = _context_order(gpulib, radii)
        got, nb = _noalloc_order(gpulib, radii)
        assert nb == len(want)
        assert np.array_equal(got[:nb], want)
        assert np.all(radii[got[nb:]] == 1e10)


def test_sort_runs_sharing_the_sorted_prefix(gpulib):
    """The digit passes sort the keys' top 24 bits; keys sharing them form runs
    that are put in full-key order afterwards.  Planted groups of radii within
    1e-12 of a centre give runs of every kind: up to 32 keys (placed by rank in
    the payload gather, or insertion-sorted by one thread in the
    allocation-free sort), hundreds (shared memory) and 5000 (in place), with
    exact ties inside them."""
    rng = np.random.default_rng(77)
    n = 60000
    radii = np.exp(rng.uniform(-6.0, 5.0, size=n))
    pos = rng.permutation(n)
    at = 0
    # 32 and 33 keys: the longest run a gather thread places and the shortest listed one
    for size, count in ((7, 400), (32, 30), (33, 30), (300, 20), (5000, 1)):
        for _ in range(count):
            c = np.exp(rng.uniform(-5.0, 4.0))
            grp = c * (1.0 + rng.uniform(0.0, 1e-12, size))
            grp[: size // 10] = grp[size // 2]  # exact ties keep input order
            radii[pos[at:at + size]] = grp
            at += size
    radii[pos[at:at + 300]] = 1e10  # escapers
    want_all = np.argsort(radii, kind="stable")
    want = want_all[radii[want_all] < 1e10]
    assert np.array_equal(_context_order(gpulib, radii), want)
    got, nb = _noalloc_order(gpulib, radii)
    assert nb == len(want) and np.array_equal(got[:nb], want)


def test_noalloc_rejects_oversize(gpulib):
    rc = gpulib.lib().cmcg_sort_radii_noalloc(C.c_void_p(16), (1 << 20) + 1, C.c_void_p(16), None, None)
    assert rc == -3  # CMCG_ERR_CAPACITY, before any device work


def test_noalloc_asynchronous_form_on_a_side_stream(gpulib):
    """Without n_bound the call only queues its work on the caller's stream;
    once that stream is synchronized the permutation is the regular sort's."""
    import torch

    rng = np.random.default_rng(99)
    n = 40000
    radii = np.exp(rng.uniform(-6.0, 5.0, size=n))
    radii[rng.random(n) < 0.02] = 1e10
    want = _context_order(gpulib, radii)
    side = torch.cuda.Stream(device="cuda:0")
    with torch.cuda.stream(side):
        d_r = torch.tensor(radii, dtype=torch.float64, device="cuda:0")
        d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda:0")
    side.synchronize()
    rc = gpulib.lib().cmcg_sort_radii_noalloc(C.c_void_p(d_r.data_ptr()), n, C.c_void_p(d_perm.data_ptr()), None,
                                             C.c_void_p(side.cuda_stream))
    assert rc == 0
    side.synchronize()
    got = d_perm.cpu().numpy().astype(np.int64)
    assert np.array_equal(got[:len(want)], want)
    assert np.all(radii[got[len(want):]] == 1e10)
