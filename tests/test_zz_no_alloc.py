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


def test_noalloc_rejects_oversize(gpulib):
    rc = gpulib.lib().cmcg_sort_radii_noalloc(C.c_void_p(16), (1 << 20) + 1, C.c_void_p(16), None, None)
    assert rc == -3  # CMCG_ERR_CAPACITY, before any device work
