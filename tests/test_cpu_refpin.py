"""The oracle pinned to the reference's own code.

oracle/ref.mk compiles the reference's Henon-step TUs (cmc_utils.c,
cmc_dynamics.c, cmc_dynamics_helper.c, cmc_evolution_thr.c, cmc_orbit.c,
cmc_nr.c, cmc_sort.c, cmc_fits.c, cmc_mpi.c, fewbody_utils.c, taus113-v2.c)
unmodified, in place, against single-rank MPI / GSL / HDF5 shims, with the
six draw sites routed to the counter generator the kernels use.  These tests
run that library (oracle.RefOracle) and the C restatement (oracle.Oracle)
side by side through the reference's main-loop phases (cmc.c:240-407) on the
benchmark configurations' models, and require every per-star field, every
global array and every step scalar to be bit-identical after every phase.

They need the reference tree, so they run where it is mounted and skip
elsewhere; tests/golden/make_refstep.py records the reference's outputs as
fixtures for the GPU tests, which run where the reference is not."""
import numpy as np
import pytest

import cmcgpu
import oracle

pytestmark = pytest.mark.skipif(oracle.reference_root() is None, reason="reference tree not present")

STAR_FIELDS = ("r", "m", "vr", "vt", "E", "J", "rnew", "vrnew", "vtnew", "rOld", "X", "Y", "r_peri", "r_apo",
               "vrold", "vtold", "Uoldrold", "Uoldrnew", "EI")
GLOBAL_ARRAYS = ("star_r", "star_m", "star_phi")
SCALARS = ("N_MAX", "N_MAX_NEW", "Mtotal", "Rtidal", "Dt", "Prev_Dt", "TotalTime", "max_r", "TidalMassLoss",
           "OldTidalMassLoss", "TidalMassLoss_old", "Eescaped", "Jescaped", "Etidal", "Etot", "KE", "PE",
           "tcount")
PHASES = ("begin_step", "calc_timestep", "dynamics_apply", "energy_conservation1", "new_orbits_calculate",
          "energy_conservation2", "tidally_strip_stars", "compute_intermediate_energy", "qsorts_new",
          "calc_potential", "energy_conservation3", "compute_energy", "end_step")


@pytest.fixture(scope="module")
def ref():
    if oracle.build_ref() is None:
        pytest.skip("reference tree not present")
    oracle.build()
    return oracle


def _differences(o, R):
    bad = []
    if not np.array_equal(o.ids(), R.ids()):
        bad.append("ids")
    for f in STAR_FIELDS + GLOBAL_ARRAYS:
        a, b = o.get(f), R.get(f)
        if a.shape != b.shape or not np.array_equal(a, b, equal_nan=True):
            n = int(np.count_nonzero(a != b)) if a.shape == b.shape else -1
            bad.append(f"{f} ({n} differ)")
    for s in SCALARS:
        a, b = o.scalar(s), R.scalar(s)
        if not (a == b or (np.isnan(a) and np.isnan(b))):
            bad.append(f"{s}: {a!r} vs {b!r}")
    return bad


def _run_phases(ic, steps, **pkw):
    """Both implementations from the same model through `steps` steps, phase
    by phase; returns the per-step total energies of each."""
    p = oracle.default_params(orbit_r=ic["rtid"], seed=20240607, **pkw)
    o = oracle.Oracle(ic, p)
    with oracle.RefOracle(ic, p) as R:
        o.initialize()
        R.initialize()
        assert not _differences(o, R), ("initialize", _differences(o, R))
        etot = []
        for step in range(steps):
            for ph in PHASES:
                if ph == "dynamics_apply":
                    o.dynamics_apply(o.scalar("Dt"))
                    R.dynamics_apply(R.scalar("Dt"))
                    continue  # Prev_Dt is set just before energy_conservation1
                if ph == "energy_conservation1":
                    o.set_scalar("Prev_Dt", o.scalar("Dt"))  # cmc.c:289; ocmc_step does the same
                    o.energy_conservation1()
                    R.energy_conservation1()
                else:
                    getattr(o, ph)()
                    getattr(R, ph)()
                bad = _differences(o, R)
                assert not bad, (step, ph, bad)
            etot.append((o.scalar("Etot"), R.scalar("Etot")))
        o.close()
    return etot


def test_reference_library_loads(ref):
    L = oracle.ref_lib()
    assert L.cmcref_sizeof_star() > 300  # star_t, include/cmc/cmc.h:409-601
    assert oracle.REF_LIB.endswith("libcmcref.so")


def test_plummer_config1_every_phase_bit_identical(ref):
    """Plummer sphere, N = 1e5 equal masses (the CPU-runnable configuration)."""
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 100_000, seed=11)
    _run_phases(ic, steps=3)


def test_king_kroupa_config2_every_phase_bit_identical(ref):
    """King W0 = 6 with Kroupa (2001) masses at the benchmark's N = 1e6."""
    ic = cmcgpu.generate(cmcgpu.KING, 1_000_000, seed=12, w0=6.0, imf=1)
    _run_phases(ic, steps=1)


def test_composite_binaries_every_phase_bit_identical(ref):
    """King W0 = 7, Kroupa masses, 10% composite binaries (the mixed-precision
    configuration's model at N = 1e5)."""
    ic = cmcgpu.generate(cmcgpu.KING, 100_000, seed=13, w0=7.0, imf=1, binary_fraction=0.1)
    _run_phases(ic, steps=3)


def test_taus113_mode_every_phase_bit_identical(ref):
    """The oracle's taus113 mode (the CPU baseline's draws) against the
    reference drawing from its own generator, one sequential stream."""
    ic = cmcgpu.generate(cmcgpu.KING, 20_000, seed=14, w0=5.0, imf=1)
    _run_phases(ic, steps=4, draw_mode=oracle.DRAW_TAUS113)


def test_energy_trajectory_over_ten_steps(ref):
    """Config 1's ten steps through the whole-step entry points: the total
    energy after every step is the reference's, bit for bit."""
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 100_000, seed=15)
    p = oracle.default_params(orbit_r=ic["rtid"], seed=99)
    o = oracle.Oracle(ic, p)
    with oracle.RefOracle(ic, p) as R:
        o.initialize()
        R.initialize()
        for _ in range(10):
            o.step()
            R.step()
            assert o.scalar("Etot") == R.scalar("Etot")
            assert o.nstars() == R.nstars()
        assert not _differences(o, R)
    o.close()


def test_potential_lookup_matches(ref):
    ic = cmcgpu.generate(cmcgpu.KING, 20_000, seed=16, w0=6.0, imf=1)
    p = oracle.default_params(orbit_r=ic["rtid"], seed=5)
    o = oracle.Oracle(ic, p)
    with oracle.RefOracle(ic, p) as R:
        o.initialize()
        R.initialize()
        rs = o.get("star_r")
        for r in np.concatenate([[0.0, 1e-6], rs[1:2000:37], rs[1:-1:977] * 1.0000001, [50.0, 1e3]]):
            assert o.potential(float(r)) == R.potential(float(r))
    o.close()


def test_nan_mass_stops_both_at_the_same_star(ref):
    """A NaN mass: the reference stops in potential_calculate (cmc_utils.c:688,
    exit_cleanly) and the oracle reports the same error there."""
    ic = cmcgpu.generate(cmcgpu.PLUMMER, 5_000, seed=17)
    p = oracle.default_params(orbit_r=ic["rtid"], seed=5)
    o = oracle.Oracle(ic, p)
    with oracle.RefOracle(ic, p) as R:
        o.initialize()
        R.initialize()
        m = o.get("star_m")
        m[1234] = np.nan
        o.set("star_m", m)
        R.set("star_m", m)
        with pytest.raises(oracle.OracleError) as eo:
            o.calc_potential()
        assert eo.value.index == 1234
        with pytest.raises(oracle.OracleError):
            R.calc_potential()
        assert R.nstars() == -1  # the reference's exit_cleanly freed its state
    o.close()


def test_golden_refstep_fixtures_are_the_references_output(ref):
    """tests/golden/refstep_*.npz (the GPU tests' inputs and expected values)
    equal what the reference's step produces now."""
    import importlib.util
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_refstep.py")
    spec = importlib.util.spec_from_file_location("make_refstep", path)
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    for case in mk.CASES:
        rec = mk.record(case)
        z = np.load(mk.path_of(case[0]))
        assert sorted(z.files) == sorted(rec), case[0]
        for k, v in rec.items():
            assert np.array_equal(z[k], np.asarray(v)), (case[0], k)
