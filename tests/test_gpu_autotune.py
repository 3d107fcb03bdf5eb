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
    assert b.variant("orbit") == 1 and b.variant("relax") == 1
    for g in (a, b):
        g.step(3)
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
    assert "orbit:" in rep and "relax:" in rep and "->" in rep, rep
    assert b.variant("orbit") in (0, 1) and b.variant("relax") in (0, 1)
    # two tunables x two variants x (one untimed + one timed step)
    a.step(8)
    a.check_device("plain")
    b.check_device("tuned")
    _same_state(a, b)
    with pytest.raises(cmcgpu.CmcError):
        b.set_variant("orbit", 2)
    with pytest.raises(KeyError):
        b.variant("nonexistent")
