"""Phase-by-phase parity of the sm_103a kernels against the CPU oracle.

Each test brings the GPU context to the oracle's exact state, runs one phase
on both, and compares: bit-exact where the arithmetic is a fixed sequence of
IEEE operations (sort permutation, pairing, time step), within the stated
relative tolerances elsewhere (see parity_util)."""
import numpy as np
import pytest

import cmcgpu
from parity_util import TOL_ORBIT, TOL_PHI, TOL_SIGMA, TOL_SUM, make_pair, max_rel, rel_err, sync_state

pytestmark = pytest.mark.gpu

CASES = [
    pytest.param(cmcgpu.PLUMMER, 6000, 0, id="plummer-eq"),
    pytest.param(cmcgpu.KING, 6000, 1, id="king6-kroupa"),
    pytest.param(cmcgpu.PLUMMER, 4001, 1, id="plummer-kroupa-odd"),
]


def _init(model, N, imf):
    ic, o, g = make_pair(model, N, seed=N + imf, imf=imf)
    o.initialize()
    g.initialize()
    return ic, o, g


@pytest.mark.parametrize("model,N,imf", CASES)
def test_potential(gpulib, orc, model, N, imf):
    ic, o, g = _init(model, N, imf)
    # the replay of potential_calculate's three FP64 recurrences is exact
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    assert g.scalar("Mtotal") == o.scalar("Mtotal")
    assert g.scalar("phi_fallback") == 0
    assert max_rel(g.scalar("Rtidal"), o.scalar("Rtidal")) <= TOL_PHI  # pow() of libm vs CUDA
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    assert max_rel(g.get("J"), o.get("J")) <= TOL_PHI
    for s in ("KE", "PE", "Etot"):
        assert max_rel(g.scalar(s), o.scalar(s)) <= TOL_SUM
    for r in (0.0, 1e-3, 0.5, 3.0, 1e3):
        assert max_rel(g.potential(r), o.potential(r)) <= TOL_PHI


@pytest.mark.parametrize("model,N,imf", CASES)
def test_timestep_and_dynamics(gpulib, orc, model, N, imf):
    ic, o, g = _init(model, N, imf)
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    g.calc_timestep()
    assert g.scalar("Dt") == o.scalar("Dt")  # bit-exact: same sums in the same order
    dt = o.scalar("Dt")
    o.dynamics_apply(dt)
    g.dynamics_apply(dt)
    g.check_device("dynamics_apply")
    assert np.array_equal(g.get("Y"), o.get("Y"))  # pairing and draws
    # velocity components against the star's speed: libm's sin/cos in the
    # deflection differ from CUDA's by an ulp, which a component near zero
    # would otherwise turn into a large relative error
    vro, vto = o.get("vr"), o.get("vt")
    speed = np.sqrt(vro * vro + vto * vto)
    assert np.max(np.abs(g.get("vr_rel") - vro) / speed) <= TOL_PHI
    assert np.max(np.abs(g.get("vt_rel") - vto) / speed) <= TOL_PHI
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    assert max_rel(g.get("J"), o.get("J")) <= TOL_PHI
    n = o.nstars()
    assert max_rel(g.get("sigma")[1:n + 1], o.get("sigma")[1:n + 1]) <= TOL_SIGMA
    assert np.array_equal(g.get("sigma_r")[1:n + 1], o.get("sigma_r")[1:n + 1])
    assert g.scalar("Nrel") == o.scalar("Nrel")
    for i in range(4):
        assert g.scalar(f"Nrelbeta{i}") == o.scalar(f"Nrelbeta{i}")


@pytest.mark.parametrize("model,N,imf", CASES[:2])
def test_dynamics_with_sines_on_the_fp32_pipe(gpulib, orc, model, N, imf):
    """cmcg_params.relax_trig32: the FP64 relaxation with its sines and
    cosines in double-float on the FP32 pipe (cmcg_fftrig.cuh).  The pairing
    draws are the oracle's bits and every output is within the relaxation's
    tolerance of the FP64 oracle (libm sin/cos): velocities against the
    star's speed, E and J at 1e-12."""
    ic = cmcgpu.generate(model, N, seed=N + imf, w0=6.0, imf=imf)
    o = orc.Oracle(ic, orc.default_params(orbit_r=ic["rtid"], seed=12345))
    g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=12345, relax_trig32=1))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    o.initialize()
    g.initialize()
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    g.calc_timestep()
    assert g.scalar("Dt") == o.scalar("Dt")
    dt = o.scalar("Dt")
    o.dynamics_apply(dt)
    g.dynamics_apply(dt)
    g.check_device("dynamics_apply")
    assert np.array_equal(g.get("Y"), o.get("Y"))
    vro, vto = o.get("vr"), o.get("vt")
    speed = np.sqrt(vro * vro + vto * vto)
    ev = max(np.max(np.abs(g.get("vr_rel") - vro) / speed), np.max(np.abs(g.get("vt_rel") - vto) / speed))
    eE, eJ = max_rel(g.get("E"), o.get("E")), max_rel(g.get("J"), o.get("J"))
    print(f"\nFP32-pipe sines: max error against the speed {ev:.2e}, E {eE:.2e}, J {eJ:.2e}")
    assert ev <= TOL_PHI and eE <= TOL_PHI and eJ <= TOL_PHI
    g.close()
    o.close()


@pytest.mark.parametrize("model,N,imf", CASES[:2])
def test_dynamics_fp32_kinematics_error(gpulib, orc, model, N, imf):
    """FP32 relaxation kinematics with FP64 energies: the error of each output
    against the FP64 oracle, relative to the star's speed (velocities) or value;
    the velocity dispersion of the sliding windows (calc_sigma_r) too."""
    ic, o, g = _init(model, N, imf)
    g32 = gpulib.Context([N], gpulib.default_params(orbit_r=ic["rtid"], seed=12345, relax_fp32=1))
    g32.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g32.initialize()
    sync_state(o, g32, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    o.calc_timestep()
    dt = o.scalar("Dt")
    o.dynamics_apply(dt)
    g32.dynamics_apply(dt)
    g32.check_device("fp32 dynamics")
    vro, vto = o.get("vr"), o.get("vt")
    speed = np.sqrt(vro * vro + vto * vto)
    err_v = max(np.max(np.abs(g32.get("vr_rel") - vro) / speed), np.max(np.abs(g32.get("vt_rel") - vto) / speed))
    err_E = max_rel(g32.get("E"), o.get("E"))
    err_J = np.max(np.abs(g32.get("J") - o.get("J")) / (o.get("star_r")[1:N + 1] * speed))
    # the window's velocity dispersion, summed in float with FP32 kinematics
    err_s = max_rel(g32.get("sigma")[1:N + 1], o.get("sigma")[1:N + 1])
    print(f"\nFP32 kinematics against FP64: v {err_v:.2e} of the speed, E {err_E:.2e}, J {err_J:.2e}, "
          f"sigma {err_s:.2e}")
    # measured on the GB300: velocities ~2e-6 of the speed, E ~3e-6 (FP32
    # deflection of nearly parallel velocities); the bound holds them to 1e-5
    assert err_v <= 1e-5 and err_E <= 1e-5 and err_J <= 1e-5 and err_s <= 1e-5, (err_v, err_E, err_J, err_s)
    assert np.array_equal(g32.get("sigma_r")[1:N + 1], o.get("sigma_r")[1:N + 1])
    assert np.array_equal(g32.get("Y"), o.get("Y"))
    g32.close()


def _to_orbits(model, N, imf):
    ic, o, g = _init(model, N, imf)
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    dt = o.scalar("Dt")
    o.dynamics_apply(dt)
    o.energy_conservation1()
    # GPU starts the orbit phase from the oracle's post-relaxation state
    sync_state(o, g, star=[("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J")],
               scalars=("Rtidal", "Mtotal"))
    o.new_orbits_calculate()
    o.energy_conservation2()
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    return ic, o, g


@pytest.mark.parametrize("model,N,imf", CASES)
def test_new_orbits(gpulib, orc, model, N, imf):
    ic, o, g = _to_orbits(model, N, imf)
    rn_o, rn_g = o.get("rnew"), g.get("rnew")
    esc_o, esc_g = rn_o == 1e10, rn_g == 1e10
    assert np.array_equal(esc_o, esc_g)
    keep = ~esc_o
    assert max_rel(rn_g[keep], rn_o[keep]) <= TOL_ORBIT
    assert max_rel(g.get("vrnew")[keep], o.get("vrnew")[keep]) <= TOL_ORBIT
    assert max_rel(g.get("vtnew")[keep], o.get("vtnew")[keep]) <= TOL_ORBIT
    # peri/apocentre and the accepted X where an orbit was sampled this step
    sampled = keep & (o.get("r_apo") > 0)
    assert max_rel(g.get("r_peri")[sampled], o.get("r_peri")[sampled]) <= TOL_ORBIT
    assert max_rel(g.get("r_apo")[sampled], o.get("r_apo")[sampled]) <= TOL_ORBIT
    assert np.array_equal(g.get("X")[sampled], o.get("X")[sampled])
    # energy_conservation1/2 folded into ec_pre
    vro, vto = o.get("vrold"), o.get("vtold")
    ec = (vto * vto + vro * vro) + 1.0 * (o.get("Uoldrold") - o.get("Uoldrnew"))
    assert max_rel(g.get("ec_pre")[keep], ec[keep]) <= TOL_ORBIT
    for s in ("TidalMassLoss", "Eescaped", "Jescaped"):
        assert max_rel(g.scalar(s), o.scalar(s)) <= 1e-10
    assert max_rel(g.scalar("max_r"), o.scalar("max_r")) <= TOL_ORBIT


@pytest.mark.parametrize("model,N,imf", CASES)
def test_tidal_sort_potential_ec3_energy(gpulib, orc, model, N, imf):
    ic, o, g = _to_orbits(model, N, imf)
    # identical inputs for the tail of the step: the oracle's orbit outputs
    sync_state(o, g, star=[("rnew", "rnew"), ("vrnew", "vrnew"), ("vtnew", "vtnew"), ("E", "E"), ("J", "J"),
                           ("r_apo", "r_apo")],
               scalars=("TidalMassLoss", "OldTidalMassLoss", "Mtotal"))
    vro, vto = o.get("vrold"), o.get("vtold")
    g.set("ec_pre", (vto * vto + vro * vro) + 1.0 * (o.get("Uoldrold") - o.get("Uoldrnew")))
    o.tidally_strip_stars()
    g.tidally_strip_stars()
    g.check_device("tidally_strip_stars")
    assert np.array_equal(g.get("rnew") == 1e10, o.get("rnew") == 1e10)
    assert max_rel(g.scalar("Rtidal"), o.scalar("Rtidal")) <= TOL_PHI
    # sort: bit-exact permutation and payload
    o.compute_intermediate_energy()
    o.qsorts_new()
    g.qsorts_new()
    g.check_device("qsorts_new")
    assert g.nstars() == o.nstars()
    assert np.array_equal(g.ids(), o.ids())
    for gn, on in (("r", "r"), ("m", "m"), ("vr", "vr"), ("vt", "vt"), ("rOld", "rOld")):
        assert np.array_equal(g.get(gn), o.get(on)), gn
    # potential of the new order: bit-exact
    o.calc_potential()
    g.calc_potential()
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    # set_velocities3 from the same potential
    sync_state(o, g, fields=("star_phi",))
    o.energy_conservation3()
    g.energy_conservation3()
    g.check_device("energy_conservation3")
    assert max_rel(g.get("vr"), o.get("vr")) <= TOL_PHI
    assert max_rel(g.get("vt"), o.get("vt")) <= TOL_PHI
    o.compute_energy()
    sync_state(o, g, scalars=("Eescaped", "Jescaped", "Etidal"))
    g.set_scalar("Eescaped_old", 0.0)
    g.set_scalar("Jescaped_old", 0.0)
    g.set_scalar("Etidal_old", 0.0)
    g.compute_energy()
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    assert max_rel(g.get("J"), o.get("J")) <= TOL_PHI
    assert max_rel(g.scalar("Etot"), o.scalar("Etot")) <= TOL_SUM


def _ec3_planted(model, N, imf, picks, d):
    """The tail of a step (stripping, sort, potential, set_velocities3) after
    making the predictions of the stars at `picks` unphysical: with
    Uoldrnew = Uoldrold + vold^2 + d, vnew^2 is about -d, and the star's excess
    0.5 (v^2 - vnew^2) m is handed on to the stars after it (the larger d,
    the further it reaches)."""
    ic, o, g = _to_orbits(model, N, imf)
    sync_state(o, g, star=[("rnew", "rnew"), ("vrnew", "vrnew"), ("vtnew", "vtnew"), ("E", "E"), ("J", "J"),
                           ("r_apo", "r_apo")],
               scalars=("TidalMassLoss", "OldTidalMassLoss", "Mtotal"))
    vro, vto = o.get("vrold"), o.get("vtold")
    vold2 = vto * vto + vro * vro
    uo, un = o.get("Uoldrold"), o.get("Uoldrnew").copy()
    un[picks] = uo[picks] + vold2[picks] + d
    o.set("Uoldrnew", un)
    g.set("ec_pre", vold2 + 1.0 * (uo - un))
    o.tidally_strip_stars()
    g.tidally_strip_stars()
    o.compute_intermediate_energy()
    o.qsorts_new()
    g.qsorts_new()
    o.calc_potential()
    g.calc_potential()
    sync_state(o, g, fields=("star_phi",))
    o.energy_conservation3()
    g.energy_conservation3()
    g.check_device("energy_conservation3")
    return o, g


def test_excess_energy_carried_across_listed_stars(gpulib, orc):
    """Listed stars close enough together that one's excess is still left when
    the walk reaches the next: the segments' carries must chain exactly as
    the sequential loop's running excess does."""
    N = 6000
    rng = np.random.default_rng(7)
    scattered = rng.choice(np.arange(1, N + 1), 200, replace=False)
    runs = np.concatenate([np.arange(s, s + 12) for s in (500, 2600, 4100)])  # adjacent listed stars
    picks = np.unique(np.concatenate([scattered, runs]))
    d = np.where(np.isin(picks, runs), 60.0, rng.uniform(0.5, 8.0, len(picks)))
    o, g = _ec3_planted(cmcgpu.PLUMMER, N, 1, picks, d)
    assert g.scalar("n_excess") >= 0.9 * len(picks)
    assert max_rel(g.get("vr"), o.get("vr")) <= TOL_PHI
    assert max_rel(g.get("vt"), o.get("vt")) <= TOL_PHI
    assert np.array_equal(g.get("vr") == 0.0, o.get("vr") == 0.0)


def test_excess_energy_beyond_the_list_capacity(gpulib, orc):
    """More unphysical predictions than the per-cluster list holds (4096): the
    whole sequential loop is replayed instead."""
    N = 12000
    rng = np.random.default_rng(11)
    picks = rng.choice(np.arange(1, N + 1), 4700, replace=False)
    o, g = _ec3_planted(cmcgpu.PLUMMER, N, 1, picks, rng.uniform(0.2, 3.0, len(picks)))
    assert g.scalar("n_excess") > 4096
    assert max_rel(g.get("vr"), o.get("vr")) <= TOL_PHI
    assert max_rel(g.get("vt"), o.get("vt")) <= TOL_PHI


@pytest.mark.parametrize("model,N,imf", CASES[:2])
def test_free_running_steps(gpulib, orc, model, N, imf):
    """Whole steps with no state injection: the same stars in the same order,
    positions that stay together, and the oracle's per-step energy change.

    The trajectories are not bit-identical: the deflection angles go through
    libm's sin/cos in the oracle and CUDA's sincos on the GPU, which differ by
    an ulp for ~20% of pairs (step 0: |dv| <= 4.4e-16, r identical to 8e-15).
    From step 1 on the time step sums see those differences, every pair
    deflects with a slightly different dt, and apsides of near-circular orbits
    amplify it.  Measured on the GB300 (r relative error, step 3 / plummer-eq,
    king6): 99th percentile 3.1e-10 / 2.0e-11, maximum 9.2e-9 / 3.1e-10.  The
    bounds hold the bulk to 1e-9 and every star to 1e-7."""
    ic, o, g = _init(model, N, imf)
    e0o, e0g = o.scalar("Etot"), g.scalar("Etot")
    for step in range(4):
        o.step()
        g.step()
        g.check_device(f"step {step}")
        assert g.nstars() == o.nstars()
        assert np.array_equal(g.ids(), o.ids())
        err = rel_err(g.get("r"), o.get("r"))
        assert np.quantile(err, 0.99) <= 1e-9 and err.max() <= 1e-7, (step, np.quantile(err, 0.99), err.max())
        de_o = o.scalar("Etot") - e0o
        de_g = g.scalar("Etot") - e0g
        assert abs(de_g - de_o) <= 1e-9 * abs(e0o) + 1e-3 * abs(de_o)


@pytest.mark.parametrize("model,N,imf", CASES)
def test_potential_replay_matches_sequential_loop(gpulib, orc, model, N, imf):
    """The parallel replay and the one-thread loop give the same bits."""
    ic, o, g = _init(model, N, imf)
    gs = gpulib.Context([N], gpulib.default_params(orbit_r=ic["rtid"], seed=12345, phi_sequential=1))
    gs.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    gs.initialize()
    assert gs.scalar("phi_fallback") == 1 and g.scalar("phi_fallback") == 0
    assert np.array_equal(g.get("star_phi"), gs.get("star_phi"))
    assert gs.scalar("Mtotal") == g.scalar("Mtotal")
    # a handful of sequential points per binade crossed, far below the record capacity
    for c in (1, 2, 3):
        assert 2 <= g.scalar(f"phi_nsp{c}") <= 200
    gs.close()


def test_potential_out_of_order_radii_fall_back(gpulib, orc):
    """Radii out of order (a host upload that skipped the sort) are outside
    the replay's proof; the cluster falls back to the one-thread loop and
    still returns the reference's bits."""
    ic, o, g = _init(cmcgpu.KING, 6000, 1)
    r = o.get("star_r").copy()
    r[100], r[101] = r[101], r[100]
    o.set("star_r", r)
    g.set("star_r", r)
    o.calc_potential()
    g.calc_potential()
    assert g.scalar("phi_fallback") == 1
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))


def test_potential_nan_mass_is_reported(gpulib, orc):
    """A NaN mass stops the potential with the reference's error (cmc_utils.c:688)
    at the same star."""
    ic, o, g = _init(cmcgpu.PLUMMER, 4001, 1)
    m = o.get("star_m").copy()
    m[1234] = np.nan
    o.set("star_m", m)
    g.set("star_m", m)
    with pytest.raises(orc.OracleError) as eo:
        o.calc_potential()
    g.calc_potential()
    code, idx = g.last_error()
    assert code == cmcgpu.CMCG_ERR_NAN_MASS == eo.value.code
    assert idx == eo.value.index == 1234


def _run_steps(gpulib, ic, N, chunks, graph):
    g = gpulib.Context([N], gpulib.default_params(orbit_r=ic["rtid"], seed=4242))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    if graph:
        g.use_graph(True)
    for k in chunks:
        g.step(k)
    g.check_device("steps")
    out = {k: g.get(k) for k in ("r", "m", "vr", "vt", "E", "J", "star_phi")}
    out["ids"] = g.ids()
    out["Etot"] = g.scalar("Etot")
    out["Rtidal"] = g.scalar("Rtidal")
    g.close()
    return out


@pytest.mark.parametrize("strip", [1, 0])
def test_whole_steps_equal_the_phase_calls(gpulib, strip):
    """Whole steps (cmcg_step) against the same steps made of the phase entry
    points in the main loop's order (cmcg_begin_step ... cmcg_compute_energy),
    with tidal stripping on (a King model that strips stars at once, so escapers
    go through the sort) and off: three steps each way, bit-identical."""
    N = 20000
    ic = cmcgpu.generate(cmcgpu.KING, N, seed=91, w0=6.0, imf=1)
    ctx = []
    for _ in range(2):
        p = cmcgpu.default_params(orbit_r=ic["rtid"] * 0.6, seed=91, TIDALLY_STRIP_STARS=strip)
        g = cmcgpu.Context([N], p)
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        ctx.append(g)
    a, b = ctx
    a.step(3)
    a.check_device("steps")
    for step in range(3):
        if step:
            b.end_step()
        b.begin_step()
        b.calc_timestep()
        b.dynamics_apply()
        b.new_orbits_calculate()
        b.tidally_strip_stars()
        b.qsorts_new()
        b.calc_potential()
        b.energy_conservation3()
        b.compute_energy()
    b.end_step()
    b.check_device("phases")
    assert a.nstars() == b.nstars()
    if strip:
        assert a.nstars() < N  # stars were stripped: escapers went through the sort
    assert np.array_equal(a.ids(), b.ids())
    for name in ("r", "m", "phi", "vr", "vt", "E", "J"):
        assert np.array_equal(a.get(name), b.get(name)), name
    for sname in ("Etot", "Mtotal", "TidalMassLoss", "max_r", "Dt"):
        assert a.scalar(sname) == b.scalar(sname), sname
    a.close()
    b.close()


def test_graph_replay_equals_direct_launches_and_is_deterministic(gpulib):
    """Steps replayed from the captured CUDA graphs (cooperative tidal launch
    included) give the same bits as direct launches, and a run repeats
    exactly (no order-dependent atomics in any result).  The graph run mixes
    single direct steps with two-step replays, so both sort-buffer parities
    get their own capture."""
    N = 20000
    ic = gpulib.generate(cmcgpu.KING, N, seed=5, imf=1)
    a = _run_steps(gpulib, ic, N, [7], graph=False)
    b = _run_steps(gpulib, ic, N, [1, 2, 1, 2, 1], graph=True)
    c = _run_steps(gpulib, ic, N, [3, 4], graph=False)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


def test_tidal_stripping_iterates_to_a_fixed_point(gpulib, orc):
    """A tidal radius cut well inside the cluster strips stars over several
    passes; the result equals the oracle's iteration."""
    ic, o, g = _to_orbits(cmcgpu.KING, 6000, 1)
    sync_state(o, g, star=[("rnew", "rnew"), ("vrnew", "vrnew"), ("vtnew", "vtnew"), ("E", "E"), ("J", "J"),
                           ("r_apo", "r_apo")],
               scalars=("TidalMassLoss", "OldTidalMassLoss"))
    # a small orbit radius puts the tidal boundary inside the cluster
    for x in (o, g):
        x.set_scalar("orbit_r", 3.0)
        x.set_scalar("Mtotal", o.scalar("Mtotal"))
    o.tidally_strip_stars()
    g.tidally_strip_stars()
    g.check_device("tidally_strip_stars")
    assert g.scalar("tidal_iters") >= 2
    assert np.array_equal(g.get("rnew") == 1e10, o.get("rnew") == 1e10)
    assert max_rel(g.scalar("Rtidal"), o.scalar("Rtidal")) <= TOL_PHI
    assert max_rel(g.scalar("TidalMassLoss"), o.scalar("TidalMassLoss")) <= 1e-10


@pytest.mark.parametrize("model,N,imf", CASES[:2])
def test_potential_queries_through_the_radius_index(gpulib, orc, model, N, imf):
    """potential(r) through the bucketed radius index equals the oracle's
    full binary search bit for bit: at table radii, their neighbours in the
    last bit, midpoints, random radii, and both ends of the table."""
    ic, o, g = _init(model, N, imf)
    r = o.get("star_r")[1:N + 1]
    rng = np.random.default_rng(11)
    pick = rng.choice(N, 300, replace=False)
    xs = list(r[pick]) + list(np.nextafter(r[pick], np.inf)) + list(np.nextafter(r[pick], 0.0))
    inner = pick[pick < N - 1]
    xs += list(0.5 * (r[inner] + r[inner + 1]))
    xs += list(np.exp(rng.uniform(np.log(r[0]), np.log(r[-1]), 300)))
    xs += [r[0], r[-1], np.nextafter(r[-1], np.inf), 0.5 * r[0], 2.0 * r[-1]]
    for x in xs:
        assert g.potential(float(x)) == o.potential(float(x)), x


@pytest.mark.parametrize("model,N,imf", CASES[:2])
def test_new_orbits_when_q_is_negative_at_the_star(gpulib, orc, model, N, imf):
    """Stars whose Q(r_j) <= 0 take get_positive_Q_index's scan from the centre
    (cmc_orbit.c:30-59); on the GPU the scan is spread over the grid.  E is
    lowered by vr^2 for a few stars so that Q(r_j) ~ -vr^2 < 0; the new orbits
    must equal the oracle's."""
    ic, o, g = _init(model, N, imf)
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    dt = o.scalar("Dt")
    o.dynamics_apply(dt)
    o.energy_conservation1()
    vr = o.get("vr")
    E = o.get("E").copy()
    pick = np.argsort(-np.abs(vr))[:6]
    E[pick] -= vr[pick] ** 2
    o.set("E", E)
    sync_state(o, g, star=[("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J")],
               scalars=("Rtidal", "Mtotal"))
    o.new_orbits_calculate()
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    rn_o, rn_g = o.get("rnew"), g.get("rnew")
    assert np.array_equal(rn_o == 1e10, rn_g == 1e10)
    keep = rn_o != 1e10
    assert max_rel(rn_g[keep], rn_o[keep]) <= TOL_ORBIT
    assert max_rel(g.get("r_peri")[pick], o.get("r_peri")[pick]) <= TOL_ORBIT
    assert max_rel(g.get("r_apo")[pick], o.get("r_apo")[pick]) <= TOL_ORBIT


def test_sign_stages_agree_near_roots(gpulib):
    """Every stage of the apsis sign test that decides agrees with the
    double-double evaluation, on points placed at relative distances 1e-18 to
    1e-2 from a root of function_q; the float-float stage decides every point
    farther than 2^-36 of the magnitudes involved."""
    rng = np.random.default_rng(5)
    n = 400000
    invN = 1.0 / 1e6
    E = -rng.uniform(0.01, 3.0, n)
    J = 10 ** rng.uniform(-4, 0.5, n)
    rj = 10 ** rng.uniform(-3, 1.7, n)
    mj = 10 ** rng.uniform(-1, 1.7, n)
    rk = 10 ** rng.uniform(-3, 1.7, n)
    phis = np.where(rk >= rj, mj * invN / rk, (mj / rj) * invN)
    B = (J / rk) ** 2
    phi0 = E - phis - 0.5 * B                 # function_q = 2 (E - Phi - phis) - (J/r)^2 = 0
    scale = np.abs(E) + np.abs(phi0) + phis + 0.5 * B
    delta = rng.choice([-1.0, 1.0], n) * 10 ** rng.uniform(-18, -2, n)
    out = cmcgpu.sign_stages(E, J, rj, mj, invN, rk, phi0 + delta * scale)
    dd = out[:, 3]
    assert (dd != 0).mean() > 0.99
    for s in range(3):
        decided = out[:, s] != 0
        wrong = decided & (out[:, s] != dd)
        assert not wrong.any(), (s, np.flatnonzero(wrong)[:5])
    far = np.abs(delta) > 2.0 ** -36
    assert (out[far, 1] != 0).all()
    # the r = 1e-20 sentinel: (J/r)^2 overflows the float stages
    m = 2000
    out0 = cmcgpu.sign_stages(E[:m], J[:m], rj[:m], mj[:m], invN, np.full(m, 1e-20), phi0[:m])
    assert (out0[:, 3] == -1).all() and (out0[:, 0] == -1).all()


@pytest.mark.parametrize("model,N", [(cmcgpu.KING, 200000), (cmcgpu.PLUMMER, 100000)])
def test_trial_filter_decisions_match_exact(gpulib, model, N):
    """With check_filters every certified FP32 accept/reject of an orbit trial
    is also evaluated exactly: whole steps run without a disagreement, and
    the state is the same as without the check."""
    ic = cmcgpu.generate(model, N, seed=3, imf=1)
    states = []
    for check in (1, 0):
        p = cmcgpu.default_params(orbit_r=ic["rtid"], seed=99, check_filters=check)
        g = cmcgpu.Context([N], [p])
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        g.step(3)
        g.check_device("three steps")
        states.append([g.get(name) for name in ("r", "vr", "vt", "m")] + [g.ids()])
        g.close()
    for a, b in zip(*states):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("model,N,imf", [(cmcgpu.PLUMMER, 6000, 0), (cmcgpu.KING, 6000, 1)])
def test_phases_with_a_central_mass(gpulib, orc, model, N, imf):
    """A central mass (cenma.m, 5% of the cluster's) enters Mtotal, Phi_0,
    set_a_b's innermost interval, potential(r < r_1) and the energies; each
    phase still matches the oracle."""
    ic, o, g = make_pair(model, N, seed=N + 7, imf=imf, cenma_m=0.05 * N)
    o.initialize()
    g.initialize()
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    assert g.scalar("Mtotal") == o.scalar("Mtotal")
    for s in ("KE", "PE", "Etot"):
        assert max_rel(g.scalar(s), o.scalar(s)) <= TOL_SUM
    for r in (1e-4, 1e-3, 0.5, 3.0):
        assert max_rel(g.potential(r), o.potential(r)) <= TOL_PHI
    # the orbit phase from the oracle's post-relaxation state
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    o.dynamics_apply(o.scalar("Dt"))
    o.energy_conservation1()
    sync_state(o, g, star=[("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J")],
               scalars=("Rtidal", "Mtotal"))
    o.new_orbits_calculate()
    o.energy_conservation2()
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    rn_o, rn_g = o.get("rnew"), g.get("rnew")
    keep = rn_o != 1e10
    assert np.array_equal(rn_g == 1e10, ~keep)
    assert max_rel(rn_g[keep], rn_o[keep]) <= TOL_ORBIT
    assert max_rel(g.get("vrnew")[keep], o.get("vrnew")[keep]) <= TOL_ORBIT
    assert max_rel(g.get("vtnew")[keep], o.get("vtnew")[keep]) <= TOL_ORBIT
    g.close()


@pytest.mark.parametrize("label,N,pkw", [
    ("apocentre-cut", 5000, dict(TIDAL_TREATMENT=0)),
    ("no-relaxation", 5000, dict(RELAXATION=0)),
    ("no-perturbation", 5000, dict(PERTURB=0)),
    ("kernel-10", 5000, dict(AVEKERNEL=10)),
    ("small-N", 48, {}),
    ("small-odd-N", 101, {}),
])
def test_free_running_steps_with_other_parameters(gpulib, orc, label, N, pkw):
    """Whole steps under the .ini switches the benchmark leaves at their
    defaults, and at small clusters (the windows need N >= 2p + 2; below it
    the reference indexes outside the star array).  Without relaxation the
    first step's positions and potential are bit-identical (no sin/cos), and
    its velocities within an ulp (set_velocities3's scale factor is formed as
    vnew2 rsqrt(vnew2 v2)); later steps, and the runs with relaxation, stay
    within the free-running bounds of test_free_running_steps."""
    model = cmcgpu.PLUMMER if N < 1000 else cmcgpu.KING
    ic, o, g = make_pair(model, N, seed=N + 13, imf=1, **pkw)
    o.initialize()
    g.initialize()
    exact = pkw.get("RELAXATION", 1) == 0 or pkw.get("PERTURB", 1) == 0
    e0o, e0g = o.scalar("Etot"), g.scalar("Etot")
    for step in range(3):
        o.step()
        g.step()
        g.check_device(f"{label} step {step}")
        assert g.nstars() == o.nstars(), (label, step)
        assert np.array_equal(g.ids(), o.ids()), (label, step)
        if exact and step == 0:
            for name in ("r", "star_phi"):
                assert np.array_equal(g.get(name), o.get(name)), (label, step, name)
            for name in ("vr", "vt", "E", "J"):
                assert max_rel(g.get(name), o.get(name)) <= TOL_PHI, (label, step, name)
        else:
            err = rel_err(g.get("r"), o.get("r"))
            assert np.quantile(err, 0.99) <= 1e-9 and err.max() <= 1e-7, (label, step, err.max())
        de_o = o.scalar("Etot") - e0o
        de_g = g.scalar("Etot") - e0g
        assert abs(de_g - de_o) <= 1e-9 * abs(e0o) + 1e-3 * abs(de_o), (label, step)
    g.close()


@pytest.mark.parametrize("learned", [False, True])
def test_n_try_exceeded_is_reported(gpulib, learned):
    """N_TRY = 1: stars whose first trial is rejected stop the step as the
    reference's exit_cleanly does (cmc_evolution_thr.c:888-891), reported as
    CMCG_ERR_NTRY with a star index, not a hang; with the learned proposal
    such a star first goes back to the plain sampler, which then runs out."""
    N = 5000
    ic = cmcgpu.generate(cmcgpu.PLUMMER, N, seed=131)
    g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=132, n_try=1))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    if learned:
        g.mlp_init(3)
        g.set_learned(cmcgpu.LEARN_ON, 1.2)
    g.step(1)
    code, idx = g.last_error()
    assert code == 5 and 1 <= idx <= N, (code, idx)  # CMCG_ERR_NTRY
    g.close()


@pytest.mark.parametrize("seed", range(1, 9))
@pytest.mark.parametrize("model,imf", [(cmcgpu.PLUMMER, 0), (cmcgpu.KING, 1), (cmcgpu.PLUMMER, 1)])
def test_potential_and_new_orbits_bit_exact_over_seeds(gpulib, orc, seed, model, imf):
    """The potential and the whole orbit phase (escapers, new r, vr, the
    accepted X) are bit-identical to the oracle on many seeded models (the
    same inputs: the oracle's post-relaxation state)."""
    N = 3000 + 37 * seed
    ic, o, g = make_pair(model, N, seed=seed * 7 + imf, imf=imf, rng_seed=seed * 13)
    o.initialize()
    g.initialize()
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    sync_state(o, g, star=[("E", "E"), ("J", "J")])
    o.begin_step()
    g.begin_step()
    o.calc_timestep()
    o.dynamics_apply(o.scalar("Dt"))
    o.energy_conservation1()
    sync_state(o, g, star=[("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J")],
               scalars=("Rtidal", "Mtotal"))
    o.new_orbits_calculate()
    o.energy_conservation2()
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    rn_o, rn_g = o.get("rnew"), g.get("rnew")
    keep = rn_o != 1e10
    assert np.array_equal(rn_g == 1e10, ~keep)
    assert np.array_equal(rn_g[keep], rn_o[keep])
    assert np.array_equal(g.get("vrnew")[keep], o.get("vrnew")[keep])
    sampled = keep & (o.get("r_apo") > 0)
    assert np.array_equal(g.get("X")[sampled], o.get("X")[sampled])
    g.close()


def test_relaxation_sines_and_cosines(gpulib):
    """The relaxation's sines and cosines, formed on the FP32 pipe in
    double-float (cmcg_fftrig.cuh: exact reduction from the draw's bits,
    Taylor series with Dekker/Knuth error-free products and sums), against
    float64 sin and cos over the whole range: within 2e-13, where the kernels'
    outputs are held to 1e-12."""
    rng = np.random.default_rng(42)
    edges = np.array([0, 1, 2, 63, 64, 65, 2**29 - 1, 2**29, 2**29 + 1, 2**30 - 1, 2**30, 2**30 + 1, 2**31 - 1,
                      2**31, 2**31 + 1, 3 * 2**30 - 1, 3 * 2**30, 3 * 2**30 + 1, 2**32 - 1], dtype=np.uint64)
    w = np.concatenate([edges, rng.integers(0, 2**32, 400_000, dtype=np.uint64)]).astype(np.uint32)
    pio4 = np.pi / 4
    bedges = np.array([0.0, 1e-300, 1e-20, 1e-8, np.nextafter(pio4, 0), pio4, np.nextafter(pio4, 2), 1.0,
                       np.nextafter(np.pi / 2, 0), np.pi / 2])
    beta = np.concatenate([bedges, rng.uniform(0, np.pi / 2, 400_000), rng.uniform(0, 1e-3, 10_000)])
    sw, sb = cmcgpu.trig_check(w, beta)
    ang = 2 * np.pi * (w.astype(np.float64) * 2.0**-32)
    err_w = max(np.max(np.abs(sw[:, 0] - np.sin(ang))), np.max(np.abs(sw[:, 1] - np.cos(ang))))
    err_b = max(np.max(np.abs(sb[:, 0] - np.sin(beta))), np.max(np.abs(sb[:, 1] - np.cos(beta))))
    # relative where the value is small (beta near 0: sin beta ~ beta)
    small = beta < 1e-3
    rel_b = np.max(np.abs(sb[small, 0] - np.sin(beta[small])) / np.maximum(np.sin(beta[small]), 1e-300))
    print(f"\nmax |error|: draws' angles {err_w:.2e}, beta {err_b:.2e}; relative for beta < 1e-3: {rel_b:.2e}")
    assert err_w <= 2e-13 and err_b <= 2e-13 and rel_b <= 2e-13
    assert sw[0, 0] == 0.0 and sw[0, 1] == 1.0 and sb[0, 0] == 0.0 and sb[0, 1] == 1.0
    assert sb[1, 0] == 1e-300 and sb[1, 1] == 1.0  # below 2^-60: sin beta = beta, cos beta = 1
