"""CPU tests of the step diagnostics (dyn.dat, lagrad.dat): the oracle's
restatement of central_calculate, clusdyn_calculate and comp_mass_percent
against an independent numpy one, and the line formats of the C-ABI
formatters (host code: no GPU needed)."""
import ctypes as C
import math

import numpy as np
import pytest

PI = 3.14159265358979323  # include/cmc/cmc.h:62


def _np_diag(o, mass_pc):
    """cmc_utils.c:872-968, 1239-1345, 1613-1624 with Python floats, one
    operation at a time in the reference's order."""
    n = o.nstars()
    r, m = o.get("star_r"), o.get("star_m")
    vr = np.concatenate([[0.0], o.get("vr")])  # per-star fields come without the k = 0 sentinel
    vt = np.concatenate([[0.0], o.get("vt")])
    NS = o.scalar("N_STAR")
    madhoc, M = o.scalar("madhoc"), o.scalar("Mtotal")
    mm, nave = 0.0, 1
    while mm < 0.5 * M:
        mm += m[nave] / NS
        nave += 1
    J = 6
    acc = [0.0] * 6
    for i in range(1, nave + 1):
        jmin = max(i - J // 2, 1)
        jmax = jmin + J
        mrho = 0.0
        for j in range(jmin + 1, jmax):
            mrho += m[j] * madhoc
        rhoj = mrho / (4.0 / 3.0 * PI * (r[jmax] * r[jmax] * r[jmax] - r[jmin] * r[jmin] * r[jmin]))
        acc[0] += rhoj
        acc[1] += rhoj * rhoj
        acc[2] += rhoj * (vr[i] * vr[i] + vt[i] * vt[i])
        acc[3] += rhoj * r[i]
        acc[4] += (rhoj * r[i]) * (rhoj * r[i])
        acc[5] += rhoj * m[i] * madhoc
    out = {"nave": nave, "rh": r[nave], "rho": acc[1] / acc[0] * (4.0 / 5.0) * 2.0,
           "v_rms": math.sqrt(acc[2] / acc[0]), "rc": acc[3] / acc[0], "rc_nb": math.sqrt(acc[4] / acc[1])}
    mprev, mc, k_at = 0.0, 0, []
    kr = np.concatenate([[0.0], np.cumsum(0.5 * m[1:n + 1] * madhoc * vr[1:n + 1] * vr[1:n + 1])])
    for k in range(1, n + 1):
        mprev += m[k] / NS
        if mc < len(mass_pc) and mprev > mass_pc[mc] * M:
            k_at.append(k)
            mc += 1
    out["no_star_r"] = np.array(k_at, float)
    out["mass_r"] = r[np.array(k_at)]
    out["ke_rad_r"] = kr[np.array(k_at)]
    return out


@pytest.mark.parametrize("model,N,imf", [(0, 3000, 1), (1, 5000, 1), (0, 4000, 0)])
def test_oracle_diagnostics_match_numpy(orc, model, N, imf):
    import cmcgpu

    ic = cmcgpu.generate(model, N, seed=11, imf=imf)
    o = orc.Oracle(ic, orc.default_params(orbit_r=ic["rtid"], seed=5))
    o.initialize()
    pc = cmcgpu.MASS_PC
    d = o.diagnostics(pc, bh_include=1)
    ref = _np_diag(o, pc)
    assert d["nave"] == ref["nave"] and d["rh"] == ref["rh"]
    for k in ("rho", "v_rms", "rc", "rc_nb"):
        assert d[k] == pytest.approx(ref[k], rel=1e-13), k
    assert np.array_equal(d["no_star_r"], ref["no_star_r"])
    assert np.array_equal(d["mass_r"], ref["mass_r"])
    assert np.allclose(d["ke_rad_r"], ref["ke_rad_r"], rtol=1e-12, atol=0)
    assert np.all(np.diff(d["no_star_r"]) >= 1)  # at most one fraction per star


def test_one_fraction_per_star(orc):
    """A heavy innermost star passes several fractions at once; the reference
    assigns them to it and the stars after it, one each."""
    import cmcgpu

    ic = cmcgpu.generate(0, 2000, seed=3, imf=0)
    m = ic["m"].copy()
    m[np.argmin(ic["r"])] *= 40.0  # the innermost star now holds ~2% of the mass
    ic = dict(ic, m=m / m.sum())
    o = orc.Oracle(ic, orc.default_params(orbit_r=ic["rtid"], seed=5))
    o.initialize()
    d = o.diagnostics(cmcgpu.MASS_PC, bh_include=1)
    ks = d["no_star_r"]
    assert list(ks[:5]) == [1, 2, 3, 4, 5]


def test_format_lines_match_the_reference_formats(gpulib):
    import cmcgpu

    a, d = cmcgpu.Diag(), cmcgpu.Diag()
    rng = np.random.default_rng(1)
    for name, _ in cmcgpu.Diag._fields_:
        for obj in (a, d):
            if name in ("tcount", "N_MAX", "nave", "n_pc", "n_set"):
                continue
            v = getattr(obj, name)
            if isinstance(v, float):
                setattr(obj, name, float(rng.normal()) * 10.0 ** int(rng.integers(-6, 6)))
    d.tcount, d.N_MAX, d.n_pc = 17, 99123, 25
    for i, p in enumerate(cmcgpu.MASS_PC):
        d.mass_pc[i] = p
        d.mass_r[i] = float(rng.uniform(1e-3, 30))
    want = ("%.8g %.8g %ld %ld %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g "
            "%.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g\n") % (
        d.TotalTime, d.Dt, d.tcount, d.N_MAX, d.Mtotal, -2.0 * d.KE / d.PE, a.N_core, a.core_radius, d.max_r,
        d.Etot, d.KE, d.PE, 0.0, 0.0, d.E_cenma, d.Eescaped, 0.0, 0.0, d.Eoops, d.Etot + d.Eoops, d.rh, a.rho_0,
        a.rc_spitzer, a.v0_rms, a.rc_nb, 0.0, 0.0, a.N_core_nb)
    assert cmcgpu.dyn_line(a, d) == want
    assert cmcgpu.lagrad_line(d) == "%.9e " % d.TotalTime + "".join("%e " % d.mass_r[i] for i in range(25)) + "\n"
    hdr = cmcgpu.lagrad_header()
    assert hdr.startswith("# Lagrange radii [code units]\n#1:t 2:r(0.0001) 3:r(0.0003)")
    assert hdr.endswith(" 26:r(0.99)\n")
    assert cmcgpu.dyn_header().splitlines()[1].split()[:3] == ["#1:t", "#2:Dt", "#3:tcount"]
    buf = C.create_string_buffer(8)
    assert cmcgpu.lib().cmcg_format_dyn_line(C.byref(a), C.byref(d), buf, 8) == -1
