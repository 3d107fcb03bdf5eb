"""Phase-by-phase parity at the benchmark configurations' sizes.

The oracle (cmc_oracle.c, bit-identical to the reference's own compiled step,
tests/test_cpu_refpin.py) and the sm_103a kernels step the same model:
  * Plummer, N = 1e5 equal masses (the CPU-runnable configuration);
  * King W0 = 6 with Kroupa masses, N = 1e6 (the benchmark's configuration);
  * King W0 = 7 with Kroupa masses and 10% composite binaries, N = 1e6 (the
    mixed-precision configuration's model at a tenth of its N).
At these sizes the potential replay crosses more binades, the radius index
has up to 2^16 buckets and the FP32 sign table outgrows L2.  Each phase starts
from the oracle's state; the bits must agree where the arithmetic is the
reference's sequence of IEEE operations, the stated tolerances elsewhere.
The rare branches of the orbit phase (sign probes left to FP64 or
double-double, apsides from the root finder) are counted and printed.  Ten
free-running steps at N = 1e5 compare the energy bookkeeping of whole runs."""
import numpy as np
import pytest

import cmcgpu
from parity_util import TOL_ORBIT, TOL_PHI, TOL_SIGMA, TOL_SUM, make_pair, max_rel, rel_err, sync_state

pytestmark = pytest.mark.gpu

CONFIGS = [
    pytest.param(dict(model=cmcgpu.PLUMMER, N=100_000, imf=0, w0=6.0, bf=0.0), id="plummer-1e5"),
    pytest.param(dict(model=cmcgpu.KING, N=1_000_000, imf=1, w0=6.0, bf=0.0), id="king6-kroupa-1e6"),
    pytest.param(dict(model=cmcgpu.KING, N=1_000_000, imf=1, w0=7.0, bf=0.1), id="king7-binaries-1e6"),
]


def _pair(cfg, seed):
    import oracle

    ic = cmcgpu.generate(cfg["model"], cfg["N"], seed=seed, w0=cfg["w0"], imf=cfg["imf"],
                         binary_fraction=cfg["bf"])
    op = oracle.default_params(orbit_r=ic["rtid"], seed=seed + 1)
    gp = cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed + 1)
    o = oracle.Oracle(ic, op)
    g = cmcgpu.Context([cfg["N"]], gp)
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    return ic, o, g


@pytest.mark.parametrize("cfg", CONFIGS)
def test_phase_by_phase_at_benchmark_size(gpulib, orc, cfg):
    ic, o, g = _pair(cfg, seed=777 + cfg["N"] % 1000 + int(10 * cfg["bf"]))
    N = cfg["N"]
    o.initialize()
    g.initialize()
    g.check_device("initialize")
    # potential_calculate: the exact replay of the three recurrences
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    assert g.scalar("Mtotal") == o.scalar("Mtotal")
    assert g.scalar("phi_fallback") == 0
    nsp = [int(g.scalar(f"phi_nsp{c}")) for c in (1, 2, 3)]
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    # time step and relaxation
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
    assert np.max(np.abs(g.get("vr_rel") - vro) / speed) <= TOL_PHI
    assert np.max(np.abs(g.get("vt_rel") - vto) / speed) <= TOL_PHI
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    assert max_rel(g.get("J"), o.get("J")) <= TOL_PHI
    n = o.nstars()
    assert max_rel(g.get("sigma")[1:n + 1], o.get("sigma")[1:n + 1]) <= TOL_SIGMA
    # new orbits from the oracle's relaxed state
    o.set_scalar("Prev_Dt", dt)
    o.energy_conservation1()
    sync_state(o, g, star=[("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J")],
               scalars=("Rtidal", "Mtotal"))
    roots_o = o.scalar("n_root_vr")
    o.new_orbits_calculate()
    o.energy_conservation2()
    roots_o = o.scalar("n_root_vr") - roots_o
    cmcgpu.orbit_counters(reset=True)
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    rare = cmcgpu.orbit_counters(reset=True)
    assert rare["root_vr"] == roots_o
    rn_o, rn_g = o.get("rnew"), g.get("rnew")
    assert np.array_equal(rn_g == 1e10, rn_o == 1e10)
    if roots_o == 0:
        # every apsis from the closed form: the reference's bits
        for k in ("rnew", "vrnew", "vtnew"):
            assert np.array_equal(g.get(k), o.get(k)), k
    else:
        keep = rn_o != 1e10
        for k in ("rnew", "vrnew", "vtnew"):
            assert max_rel(g.get(k)[keep], o.get(k)[keep]) <= TOL_ORBIT, k
    sampled = (rn_o != 1e10) & (o.get("r_apo") > 0)
    assert np.array_equal(g.get("X")[sampled], o.get("X")[sampled])
    assert max_rel(g.get("r_peri")[sampled], o.get("r_peri")[sampled]) <= (0 if roots_o == 0 else TOL_ORBIT)
    assert max_rel(g.get("r_apo")[sampled], o.get("r_apo")[sampled]) <= (0 if roots_o == 0 else TOL_ORBIT)
    # the tail: stripping, sort, potential, set_velocities3, energies
    sync_state(o, g, star=[("rnew", "rnew"), ("vrnew", "vrnew"), ("vtnew", "vtnew"), ("E", "E"), ("J", "J"),
                           ("r_apo", "r_apo")],
               scalars=("TidalMassLoss", "OldTidalMassLoss", "Mtotal"))
    vrold, vtold = o.get("vrold"), o.get("vtold")
    g.set("ec_pre", (vtold * vtold + vrold * vrold) + 1.0 * (o.get("Uoldrold") - o.get("Uoldrnew")))
    o.tidally_strip_stars()
    g.tidally_strip_stars()
    g.check_device("tidally_strip_stars")
    assert np.array_equal(g.get("rnew") == 1e10, o.get("rnew") == 1e10)
    o.compute_intermediate_energy()
    o.qsorts_new()
    g.qsorts_new()
    g.check_device("qsorts_new")
    assert g.nstars() == o.nstars()
    assert np.array_equal(g.ids(), o.ids())
    for k in ("r", "m", "vr", "vt", "rOld"):
        assert np.array_equal(g.get(k), o.get(k)), k
    o.calc_potential()
    g.calc_potential()
    g.check_device("calc_potential")
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    assert g.scalar("phi_fallback") == 0
    o.energy_conservation3()
    g.energy_conservation3()
    g.check_device("energy_conservation3")
    assert max_rel(g.get("vr"), o.get("vr")) <= TOL_PHI
    assert max_rel(g.get("vt"), o.get("vt")) <= TOL_PHI
    o.compute_energy()
    sync_state(o, g, scalars=("Eescaped", "Jescaped", "Etidal"))
    for s in ("Eescaped_old", "Jescaped_old", "Etidal_old"):
        g.set_scalar(s, 0.0)
    g.compute_energy()
    assert max_rel(g.get("E"), o.get("E")) <= TOL_PHI
    assert max_rel(g.get("J"), o.get("J")) <= TOL_PHI
    assert max_rel(g.scalar("Etot"), o.scalar("Etot")) <= TOL_SUM
    print(f"\n[{N} stars] potential sequential points {nsp}; orbit probes decided in FP64 "
          f"{rare['sign_f64']}, in double-double {rare['sign_dd']}; apsides from the root finder "
          f"{rare['root_vr']} (oracle {int(roots_o)})")
    g.close()
    o.close()


@pytest.mark.parametrize("model,imf", [(cmcgpu.PLUMMER, 0), (cmcgpu.KING, 1)], ids=["plummer-1e5", "king6-kroupa-1e5"])
def test_ten_free_running_steps(gpulib, orc, model, imf):
    """Ten whole steps at N = 1e5 without state injection, the GPU against the
    oracle.

    The two runs part in the last bits at the first relaxation: the deflection
    angles go through libm's sin/cos in the oracle and CUDA's on the GPU.  For
    the first two steps the same stars stay in order (but for neighbours
    closer than the drift, which may trade places), radii agree to
    ~1e-10 (99th percentile, measured on the GB300: 6.8e-11 Plummer, 6.0e-11
    King) and the energy change agrees to ~1e-14 of the total.  Then an ulp of
    E moves some rejection trial across its acceptance test, that star lands
    at an unrelated radius, and from there the runs are two realisations of
    the same chaotic process: a star escapes in one and not the other by step
    3 (Plummer) or 7 (King).  The energy bookkeeping must still agree: the
    cumulative energy change of the two runs stays within a small fraction of
    the total energy (measured after ten steps: 1.2e-6 Plummer, 2.1e-5 King)."""
    cfg = dict(model=model, N=100_000, imf=imf, w0=6.0, bf=0.0)
    ic, o, g = _pair(cfg, seed=2024)
    o.initialize()
    g.initialize()
    e0o, e0g = o.scalar("Etot"), g.scalar("Etot")
    for step in range(10):
        o.step()
        g.step()
        g.check_device(f"step {step}")
        de_o = o.scalar("Etot") - e0o
        de_g = g.scalar("Etot") - e0g
        print(f"step {step}: energy change {de_g:.6e} (oracle {de_o:.6e}), stars {g.nstars()} ({o.nstars()})")
        if step < 2:
            # the same stars, each at the oracle's radius to the drift; two
            # neighbours closer than the drift may trade places in the order
            assert g.nstars() == o.nstars()
            ids_g, ids_o = g.ids(), o.ids()
            assert np.array_equal(np.sort(ids_g), np.sort(ids_o)), step
            assert np.mean(ids_g == ids_o) >= 0.999, step
            err = rel_err(g.get("r")[np.argsort(ids_g)], o.get("r")[np.argsort(ids_o)])
            assert np.quantile(err, 0.99) <= 1e-9 and err.max() <= 1e-6, (step, np.quantile(err, 0.99), err.max())
            assert abs(de_g - de_o) <= 1e-12 * abs(e0o), (step, de_g, de_o)
        else:
            assert abs(g.nstars() - o.nstars()) <= 1e-3 * o.nstars(), step
            assert abs(de_g - de_o) <= 2e-4 * abs(e0o), (step, de_g, de_o)
    g.close()
    o.close()


def test_config5_size_one_step_properties(gpulib, orc):
    """The mixed-precision configuration's model at its full size: King W0 = 7,
    Kroupa masses, 10% composite binaries, N = 1e7, FP32 relaxation
    kinematics.  The oracle steps 1e6 stars in ~8 s on one core, so at 1e7
    the whole step is checked through properties that hold at any size:
      * the initial potential, Mtotal and energies against the oracle (the
        replay at 1e7 stars crosses more binades than any smaller case);
      * after one GPU step, the radii in order, the ids a duplicate-free
        subset of the initial ones, the stars removed accounted for by the
        tidal mass loss;
      * the potential the step ends with equal, bit for bit, to the oracle's
        potential_calculate on the GPU's own post-step radii and masses, and
        potential(r) through the radius index equal to the oracle's search."""
    N = 10_000_000
    ic = cmcgpu.generate(cmcgpu.KING, N, seed=31, w0=7.0, imf=1, binary_fraction=0.1)
    seed = 4242
    op = orc.default_params(orbit_r=ic["rtid"], seed=seed)
    gp = cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed, relax_fp32=1)
    o = orc.Oracle(ic, op)
    g = cmcgpu.Context([N], gp)
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    o.initialize()
    g.initialize()
    g.check_device("initialize")
    assert np.array_equal(g.get("star_phi"), o.get("star_phi"))
    assert g.scalar("Mtotal") == o.scalar("Mtotal")
    assert g.scalar("phi_fallback") == 0
    for s in ("KE", "PE", "Etot"):
        assert max_rel(g.scalar(s), o.scalar(s)) <= TOL_SUM, s
    n_star = int(o.scalar("N_STAR"))
    m0 = g.scalar("Mtotal")
    e0 = g.scalar("Etot")
    o.close()

    g.step(1)
    g.check_device("step")
    n1 = g.nstars()
    r = g.get("r")
    assert len(r) == n1 and np.all(np.diff(r) >= 0.0)
    ids = g.ids()
    assert len(np.unique(ids)) == n1 and np.all(np.isin(ids, ic["id"]))
    m1 = g.scalar("Mtotal")
    lost = g.scalar("TidalMassLoss")
    assert 0 < n1 < N
    assert abs(m0 - (m1 + lost)) <= 1e-12 * m0, (m0, m1, lost)
    # Etot counts the escapers' energy (Eescaped, compute_energy_new); measured on the GB300:
    # -8.5e-4 of it in this first step, which strips 4% of the mass
    de = (g.scalar("Etot") - e0) / abs(e0)
    print(f"\n[{N} stars] one step: {N - n1} stars stripped, mass lost {lost:.6e}, relative change of Etot "
          f"{de:.3e} (Eescaped {g.scalar('Eescaped'):.6e}, Etidal {g.scalar('Etidal'):.6e})")
    assert abs(de) <= 1e-2

    # the oracle's potential_calculate on the GPU's post-step state
    sp = orc.default_params(orbit_r=ic["rtid"], seed=seed, N_STAR=n_star)
    mg = g.get("m")
    post = {"r": r, "m": mg / n_star, "vr": g.get("vr"), "vt": g.get("vt"), "id": ids}
    o2 = orc.Oracle(post, sp)
    o2.set("star_r", g.get("star_r"))
    o2.set("star_m", g.get("star_m"))
    o2.calc_potential()
    assert o2.nstars() == n1
    assert o2.scalar("Mtotal") == m1
    assert np.array_equal(g.get("star_phi"), o2.get("star_phi"))
    # potential(r) through the radius index (2^20 buckets at this size) against
    # the oracle's full binary search on the same table
    rng = np.random.default_rng(5)
    pick = rng.choice(n1, 200, replace=False)
    xs = list(r[pick]) + list(np.nextafter(r[pick], np.inf)) + list(np.nextafter(r[pick], 0.0))
    xs += list(np.exp(rng.uniform(np.log(r[0]), np.log(r[-1]), 200))) + [r[0], r[-1], 2.0 * r[-1]]
    for x in xs:
        assert g.potential(float(x)) == o2.potential(float(x)), x
    o2.close()
    g.close()
