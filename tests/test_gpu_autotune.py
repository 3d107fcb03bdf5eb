"""The autotuner's launch variants give bit-identical results, and tuning
steps are ordinary steps of the run."""
import numpy as np
import pytest

import cmcgpu

pytestmark = pytest.mark.gpu


def _pair(N, seed, model=cmcgpu.KING, imf=1):
    ic = cmcgpu.generate(model, N, seed=seed, imf=imf)
    out = []
    for _ in range(2):
        g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed + 1))
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        out.append(g)
    return out


def _same_state(a, b):
    for name in ("r", "vr", "vt", "m", "E", "J", "star_phi", "X", "r_peri", "r_apo"):
        assert np.array_equal(a.get(name), b.get(name)), name
    assert np.array_equal(a.ids(), b.ids())
    for s in ("Etot", "Dt", "max_r", "TotalTime"):
        assert a.scalar(s) == b.scalar(s), s


def test_plain_variants_are_bit_identical(gpulib):
    a, b = _pair(30000, 81)
    b.set_variant("orbit", 1)
    b.set_variant("relax", 1)
    b.set_variant("sort_tile", 2)    # 1024-key digit-pass tiles
    b.set_variant("gather_tile", 2)  # 1024-star gather blocks
    assert b.variant("orbit") == 1 and b.variant("relax") == 1
    for g in (a, b):
        g.step(3)
        g.check_device("steps")
    _same_state(a, b)


@pytest.mark.parametrize("variant", [2, 3])
def test_persistent_orbit_kernels_are_bit_identical(gpulib, variant):
    """The persistent orbit kernels (a grid the SMs hold, tiles taken from a
    counter) against the one-block-per-tile grid, on an ensemble of uneven
    clusters so tiles of different clusters interleave."""
    Ns = [20000, 3000, 45000]
    ics = [cmcgpu.generate(cmcgpu.KING if i % 2 else cmcgpu.PLUMMER, n, seed=90 + i, imf=1) for i, n in enumerate(Ns)]
    out = []
    for v in (0, variant):
        g = cmcgpu.Context(Ns, [cmcgpu.default_params(orbit_r=ic["rtid"], seed=7 + i) for i, ic in enumerate(ics)])
        for i, ic in enumerate(ics):
            g.load(i, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        g.set_variant("orbit", v)
        g.step(3)
        g.check_device("steps")
        out.append(g)
    a, b = out
    for c in range(len(Ns)):
        for name in ("r", "vr", "vt", "E", "J", "X", "r_peri", "r_apo"):
            assert np.array_equal(a.get(name, c), b.get(name, c)), (c, name)
        assert np.array_equal(a.ids(c), b.ids(c))
        for s in ("Etot", "max_r", "TidalMassLoss"):
            assert a.scalar(s, c) == b.scalar(s, c), (c, s)


@pytest.mark.parametrize("sort_tile,gather_tile", [(1, 1), (0, 2), (1, 0), (2, 0), (2, 1)])
def test_sort_tile_variants_are_bit_identical(gpulib, sort_tile, gather_tile):
    """The sort's tile sizes (digit pass 4096, 2048 or 1024 keys; gather blocks of
    256, 128 or 1024 stars) on a 200,000-star cluster: hundreds of tiles, so
    the look-back and the tile tables are exercised at every size."""
    a, b = _pair(200000, 87)
    b.set_variant("sort_tile", sort_tile)
    b.set_variant("gather_tile", gather_tile)
    for g in (a, b):
        g.step(2)
        g.check_device("steps")
    _same_state(a, b)


def test_learned_variants_are_bit_identical(gpulib):
    a, b = _pair(30000, 83, model=cmcgpu.PLUMMER, imf=0)
    for g in (a, b):
        g.mlp_init(3)
        g.set_learned(cmcgpu.LEARN_ON, 1.2)
    b.set_variant("orbit_learn", 1)
    b.set_variant("mlp_grid", 3)
    for g in (a, b):
        g.step(2)
        g.check_device("learned steps")
    _same_state(a, b)


def test_tuning_steps_are_steps_of_the_run(gpulib):
    a, b = _pair(30000, 85)
    rep = b.autotune(1)
    assert "orbit:" in rep and "relax:" in rep and "sort_tile:" in rep and "gather_tile:" in rep, rep
    assert b.variant("orbit") in (0, 1, 2, 3) and b.variant("relax") in (0, 1)
    assert b.variant("sort_tile") in (0, 1, 2) and b.variant("gather_tile") in (0, 1, 2)
    # orbit with four variants, relax with two, the sort tile and the gather
    # with three, each variant one untimed and one timed step
    a.step(2 * (4 + 2 + 3 + 3))
    a.check_device("plain")
    b.check_device("tuned")
    _same_state(a, b)
    with pytest.raises(cmcgpu.CmcError):
        b.set_variant("orbit", 4)
    with pytest.raises(KeyError):
        b.variant("nonexistent")
