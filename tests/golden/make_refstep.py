"""Record the reference's own Henon step as fixtures for the GPU tests.

The reference's hot-path TUs, compiled in place by oracle/ref.mk
(oracle.RefOracle), step three small models phase by phase from their initial
state.  For each phase this writes what the GPU test feeds in and what it
checks: full arrays where the kernels are held to a tolerance or need the
reference's values as inputs, SHA-256 digests of the raw float64 / int64
bytes where they must be bit-identical.

    python tests/golden/make_refstep.py        # where the reference tree is mounted

Writes tests/golden/refstep_<case>.npz; tests/test_cpu_refpin.py checks that
the files still equal what the reference produces, tests/test_gpu_refstep.py
runs the kernels against them.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for sub in ("oracle", "cmc-cosmic_gb300"):
    sys.path.insert(0, os.path.join(ROOT, sub))
import cmcgpu  # noqa: E402
import oracle  # noqa: E402

# (name, model, N, model seed, W0, IMF, composite-binary fraction, draw seed)
CASES = [
    ("plummer_eq", cmcgpu.PLUMMER, 1200, 31, 6.0, 0, 0.0, 4001),
    ("king6_kroupa", cmcgpu.KING, 1200, 32, 6.0, 1, 0.0, 4002),
    ("king7_binaries", cmcgpu.KING, 1200, 33, 7.0, 1, 0.1, 4003),
]


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def record(case) -> dict:
    """The reference's step 0 from the case's model, phase by phase."""
    name, model, N, mseed, w0, imf, bf, dseed = case
    ic = cmcgpu.generate(model, N, seed=mseed, w0=w0, imf=imf, binary_fraction=bf)
    p = oracle.default_params(orbit_r=ic["rtid"], seed=dseed)
    out = {"N": N, "draw_seed": dseed, "rtid": ic["rtid"]}
    for k in ("r", "m", "vr", "vt"):
        out["ic_" + k] = np.asarray(ic[k], np.float64)
    out["ic_id"] = np.asarray(ic["id"], np.int64)
    with oracle.RefOracle(ic, p) as R:
        R.initialize()
        out["init_phi_sha"] = digest(R.get("star_phi"))
        out["init_Mtotal"] = R.scalar("Mtotal")
        out["init_E"], out["init_J"] = R.get("E"), R.get("J")
        for s in ("KE", "PE", "Etot"):
            out["init_" + s] = R.scalar(s)
        R.begin_step()
        R.calc_timestep()
        out["Dt"] = R.scalar("Dt")
        R.dynamics_apply(R.scalar("Dt"))
        out["relax_Y_sha"] = digest(R.get("Y"))
        for k in ("vr", "vt", "E", "J"):
            out["relax_" + k] = R.get(k)
        out["relax_Rtidal"], out["relax_Mtotal"] = R.scalar("Rtidal"), R.scalar("Mtotal")
        R.energy_conservation1()
        R.new_orbits_calculate()
        R.energy_conservation2()
        for k in ("rnew", "vrnew", "vtnew"):
            out["orbit_" + k + "_sha"] = digest(R.get(k))
        for k in ("X", "r_peri", "r_apo"):  # compared where an orbit was sampled
            out["orbit_" + k] = R.get(k)
        out["orbit_escaped_sha"] = digest(R.get("rnew") == 1e10)
        for s in ("TidalMassLoss", "OldTidalMassLoss", "Eescaped", "Jescaped", "max_r"):
            out["orbit_" + s] = R.scalar(s)
        # the energy-conservation carry across the sort (set_velocities3's
        # vold^2 + 2 (1 - q)(Uoldrold - Uoldrnew) with q = 1/2), which the
        # kernels keep as one field
        vro, vto = R.get("vrold"), R.get("vtold")
        out["orbit_ec_pre"] = (vto * vto + vro * vro) + 1.0 * (R.get("Uoldrold") - R.get("Uoldrnew"))
        R.tidally_strip_stars()
        out["tidal_escaped_sha"] = digest(R.get("rnew") == 1e10)
        out["tidal_Rtidal"] = R.scalar("Rtidal")
        R.compute_intermediate_energy()
        R.qsorts_new()
        out["sort_n"] = R.nstars()
        out["sort_ids_sha"] = digest(R.ids())
        for k in ("r", "m", "vr", "vt", "rOld"):
            out["sort_" + k + "_sha"] = digest(R.get(k))
        R.calc_potential()
        out["pot_phi_sha"] = digest(R.get("star_phi"))
        out["pot_Mtotal"] = R.scalar("Mtotal")
        R.energy_conservation3()
        out["ec3_vr"], out["ec3_vt"] = R.get("vr"), R.get("vt")
        R.compute_energy()
        out["energy_E"], out["energy_J"] = R.get("E"), R.get("J")
        for s in ("Etot", "Eescaped", "Jescaped", "Etidal"):
            out["energy_" + s] = R.scalar(s)
    return out


def path_of(name: str) -> str:
    return os.path.join(HERE, f"refstep_{name}.npz")


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference tree not found; cannot record the reference's step")
    for case in CASES:
        rec = record(case)
        np.savez_compressed(path_of(case[0]), **{k: np.asarray(v) for k, v in rec.items()})
        print("wrote", path_of(case[0]), os.path.getsize(path_of(case[0])), "bytes")


if __name__ == "__main__":
    main()
