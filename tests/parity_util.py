"""Shared helpers for the GPU-vs-oracle parity tests."""
import numpy as np

import cmcgpu
import oracle

# Tolerances (relative), the bars the parity tests hold the kernels to:
TOL_PHI = 1e-12      # potential, E, J
TOL_ORBIT = 1e-9     # new r, vr, vt
TOL_SIGMA = 1e-10    # sliding-window sigma (the reference keeps a running sum)
TOL_SUM = 1e-12      # order-dependent global sums (energies, escaped energy)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), 1e-300)
    return np.where(a == b, 0.0, np.abs(a - b) / den)


def max_rel(a, b):
    e = rel_err(a, b)
    return float(e.max()) if e.size else 0.0


def make_pair(model=cmcgpu.PLUMMER, N=4000, seed=1, imf=0, w0=6.0, rng_seed=12345, **pkw):
    ic = cmcgpu.generate(model, N, seed=seed, w0=w0, imf=imf)
    op = oracle.default_params(orbit_r=ic["rtid"], seed=rng_seed, **pkw)
    gp = cmcgpu.default_params(orbit_r=ic["rtid"], seed=rng_seed, **pkw)
    o = oracle.Oracle(ic, op)
    g = cmcgpu.Context([N], gp)
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    return ic, o, g


def sync_state(o, g, fields=("star_r", "star_m", "star_phi"), star=(), scalars=()):
    """Copy the oracle's state into the GPU context (global arrays, per-star
    fields given as (oracle_name, gpu_name) pairs, scalars)."""
    for name in fields:
        g.set(name, o.get(name))
    for on, gn in star:
        g.set(gn, o.get(on))
    for s in scalars:
        g.set_scalar(s, o.scalar(s))
