"""The sm_103a kernels against the reference's own step, phase by phase.

tests/golden/refstep_<case>.npz hold what the reference's compiled Henon-step
code (oracle/ref.mk, recorded by tests/golden/make_refstep.py) does to three
small models -- Plummer with equal masses, King W0 = 6 with Kroupa masses,
King W0 = 7 with 10% composite binaries -- in the first step.  Each test loads
the same initial model, runs the GPU through the same phases, feeds in the
reference's values where the kernels are allowed to differ in the last ulps
(relaxation, through CUDA's sin/cos), and requires the reference's bits where
the arithmetic is the same sequence of IEEE operations: the potential, the
time step, the pairing draws, the new orbits, the stripping, the sort
permutation and payload, the new potential."""
import hashlib
import os

import numpy as np
import pytest

from parity_util import TOL_ORBIT, TOL_PHI, TOL_SUM, max_rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["plummer_eq", "king6_kroupa", "king7_binaries"]


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _load(name):
    z = np.load(os.path.join(GOLD, f"refstep_{name}.npz"))
    return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}


@pytest.mark.parametrize("case", CASES)
def test_step_against_the_reference(gpulib, case):
    f = _load(case)
    N = int(f["N"])
    g = gpulib.Context([N], gpulib.default_params(orbit_r=float(f["rtid"]), seed=int(f["draw_seed"])))
    g.load(0, f["ic_r"], f["ic_m"], f["ic_vr"], f["ic_vt"], f["ic_id"])

    # potential_calculate + compute_energy of the initial model
    g.initialize()
    g.check_device("initialize")
    assert digest(g.get("star_phi")) == f["init_phi_sha"]
    assert g.scalar("Mtotal") == f["init_Mtotal"]
    assert max_rel(g.get("E"), f["init_E"]) <= TOL_PHI
    assert max_rel(g.get("J"), f["init_J"]) <= TOL_PHI
    for s in ("KE", "PE", "Etot"):
        assert max_rel(g.scalar(s), f["init_" + s]) <= TOL_SUM

    # calc_timestep, dynamics_apply from the reference's energies
    g.set("E", f["init_E"])
    g.set("J", f["init_J"])
    g.begin_step()
    g.calc_timestep()
    assert g.scalar("Dt") == f["Dt"]
    g.dynamics_apply(f["Dt"])
    g.check_device("dynamics_apply")
    assert digest(g.get("Y")) == f["relax_Y_sha"]
    vro, vto = f["relax_vr"], f["relax_vt"]
    speed = np.sqrt(vro * vro + vto * vto)
    assert np.max(np.abs(g.get("vr_rel") - vro) / speed) <= TOL_PHI
    assert np.max(np.abs(g.get("vt_rel") - vto) / speed) <= TOL_PHI
    assert max_rel(g.get("E"), f["relax_E"]) <= TOL_PHI
    assert max_rel(g.get("J"), f["relax_J"]) <= TOL_PHI

    # new_orbits_calculate (get_positions) from the reference's relaxed state
    g.set("vr_rel", vro)
    g.set("vt_rel", vto)
    g.set("E", f["relax_E"])
    g.set("J", f["relax_J"])
    g.set_scalar("Rtidal", f["relax_Rtidal"])
    g.set_scalar("Mtotal", f["relax_Mtotal"])
    gpulib.orbit_counters(reset=True)
    g.new_orbits_calculate()
    g.check_device("new_orbits_calculate")
    # the reference found every apsis of these models by its closed form (its
    # Brent fallback, cmc_nr.c:500, never ran), and so must the kernels
    assert gpulib.orbit_counters(reset=True)["root_vr"] == 0
    rnew = g.get("rnew")
    assert digest(rnew == 1e10) == f["orbit_escaped_sha"]
    assert digest(rnew) == f["orbit_rnew_sha"]
    assert digest(g.get("vrnew")) == f["orbit_vrnew_sha"]
    assert digest(g.get("vtnew")) == f["orbit_vtnew_sha"]
    sampled = (rnew != 1e10) & (f["orbit_r_apo"] > 0)
    for k in ("X", "r_peri", "r_apo"):
        assert np.array_equal(g.get(k)[sampled], f["orbit_" + k][sampled]), k
    for s in ("TidalMassLoss", "Eescaped", "Jescaped"):
        assert max_rel(g.scalar(s), f["orbit_" + s]) <= 1e-10
    assert max_rel(g.scalar("max_r"), f["orbit_max_r"]) <= TOL_ORBIT

    # tidally_strip_stars, ComputeIntermediateEnergy + qsorts_new + post_sort_comm
    g.set("ec_pre", f["orbit_ec_pre"])
    g.set("r_apo", f["orbit_r_apo"])
    for s in ("TidalMassLoss", "OldTidalMassLoss"):
        g.set_scalar(s, f["orbit_" + s])
    g.tidally_strip_stars()
    g.check_device("tidally_strip_stars")
    assert digest(g.get("rnew") == 1e10) == f["tidal_escaped_sha"]
    assert max_rel(g.scalar("Rtidal"), f["tidal_Rtidal"]) <= TOL_PHI
    g.qsorts_new()
    g.check_device("qsorts_new")
    assert g.nstars() == int(f["sort_n"])
    assert digest(g.ids()) == f["sort_ids_sha"]
    for k in ("r", "m", "vr", "vt", "rOld"):
        assert digest(g.get(k)) == f["sort_" + k + "_sha"], k

    # calc_potential_new of the new order, set_velocities3, compute_energy_new
    g.calc_potential()
    g.check_device("calc_potential")
    assert digest(g.get("star_phi")) == f["pot_phi_sha"]
    assert g.scalar("Mtotal") == f["pot_Mtotal"]
    g.energy_conservation3()
    g.check_device("energy_conservation3")
    assert max_rel(g.get("vr"), f["ec3_vr"]) <= TOL_PHI
    assert max_rel(g.get("vt"), f["ec3_vt"]) <= TOL_PHI
    for s in ("Eescaped", "Jescaped", "Etidal"):
        g.set_scalar(s, f["energy_" + s])
        g.set_scalar(s + "_old", 0.0)
    g.compute_energy()
    assert max_rel(g.get("E"), f["energy_E"]) <= TOL_PHI
    assert max_rel(g.get("J"), f["energy_J"]) <= TOL_PHI
    assert max_rel(g.scalar("Etot"), f["energy_Etot"]) <= TOL_SUM
    g.close()
