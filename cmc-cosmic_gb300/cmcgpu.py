"""Python binding of libcmcgpu.so (include/cmcgpu.h) over ctypes.

This module mirrors the reference's step-level interface for tests and the
benchmark: a :class:`Context` holds one or more clusters resident on the GPU and
exposes the main-loop phases under the reference's names (``dynamics_apply``,
``new_orbits_calculate``, ``qsorts_new``, ``calc_potential`` ...).  Errors
raised on the device come back as :class:`CmcError` with the code of the
reference's ``exit_cleanly`` site they mirror.

There is no CPU fallback: constructing a Context without a usable GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcmcgpu.so")
IC_LIB_PATH = os.path.join(_HERE, "_build", "libcmcic.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "cmcgpu.h")

ERRORS = {
    -1: "bad argument", -2: "CUDA error", -3: "capacity exceeded", -4: "out of device memory",
    -5: "bad state", -6: "file not readable", -7: "file layout not read here", 1: "NaN in mass sum", 2: "NaN in potential", 3: "W = 0 in encounter",
    4: "wp = 0 in deflection", 5: "N_TRY exceeded", 6: "vr^2 is NaN", 7: "no sign change of vr^2",
    8: "apsis root not converged", 9: "negative residual at apsis", 10: "radius search failed",
    11: "radius outside interval", 12: "strong encounter drawn", 20: "bounded wait gave up",
    21: "tidal stripping did not settle",
}


CMCG_ERR_NAN_MASS, CMCG_ERR_NAN_PHI = 1, 2
CMCG_ERR_IO, CMCG_ERR_FORMAT = -6, -7


class CmcError(RuntimeError):
    def __init__(self, code: int, where: str = "", index: int = -1):
        self.code = code
        self.index = index
        super().__init__(f"{where}: {ERRORS.get(code, 'error')} (code {code}, index {index})")


class Params(C.Structure):
    _fields_ = [
        ("N_STAR", C.c_long), ("AVEKERNEL", C.c_long), ("GAMMA", C.c_double), ("THETASEMAX", C.c_double),
        ("PERTURB", C.c_int), ("RELAXATION", C.c_int), ("TIDALLY_STRIP_STARS", C.c_int),
        ("TIDAL_TREATMENT", C.c_int), ("orbit_r", C.c_double), ("cenma_m", C.c_double),
        ("apsides_max_iter", C.c_long), ("apsides_precision", C.c_double),
        ("apsides_convergence", C.c_double), ("n_try", C.c_long), ("seed", C.c_uint64),
        ("relax_fp32", C.c_int), ("phi_sequential", C.c_int), ("check_filters", C.c_int), ("relax_trig32", C.c_int),
    ]


CMCG_MASS_PC_MAX = 64
# the reference's example MASS_PC (examples/KingProfile.ini, PlummerSphere.ini)
MASS_PC = (0.0001, 0.0003, 0.0005, 0.0007, 0.0009, 0.001, 0.003, 0.005, 0.007, 0.009, 0.01, 0.03, 0.05, 0.07, 0.09,
           0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 0.99)


class Diag(C.Structure):
    """cmcg_diag (cmcgpu.h)."""
    _fields_ = ([("TotalTime", C.c_double), ("Dt", C.c_double), ("tcount", C.c_long), ("N_MAX", C.c_long)]
                + [(n, C.c_double) for n in ("Mtotal", "Etot", "KE", "PE", "E_cenma", "Eescaped", "Eoops", "max_r")]
                + [("nave", C.c_long), ("rh", C.c_double)]
                + [(n, C.c_double) for n in ("rho_0", "v0_rms", "core_radius", "rc_nb", "m_ave", "n_central",
                                            "rc_spitzer", "N_core", "N_core_nb", "Trc")]
                + [("n_pc", C.c_int), ("n_set", C.c_int)]
                + [(n, C.c_double * CMCG_MASS_PC_MAX) for n in ("mass_pc", "mass_r", "ave_mass_r", "no_star_r",
                                                                "densities_r", "ke_rad_r", "ke_tan_r", "v2_rad_r",
                                                                "v2_tan_r")])

    def arr(self, name: str):
        return np.array(getattr(self, name)[:self.n_pc])


def _fmt(fn, *args) -> str:
    buf = C.create_string_buffer(1 << 16)
    n = fn(*args, buf, len(buf))
    if n < 0:
        raise RuntimeError("format buffer too small")
    return buf.value.decode()


def dyn_header() -> str:
    return _fmt(lib().cmcg_format_dyn_header)


def lagrad_header(mass_pc=MASS_PC) -> str:
    pc = np.ascontiguousarray(mass_pc, dtype=np.float64)
    return _fmt(lib().cmcg_format_lagrad_header, pc.ctypes.data, len(pc))


def dyn_line(start: "Diag", end: "Diag") -> str:
    """dyn.dat line: core quantities from `start` (before the step), the rest from `end`."""
    return _fmt(lib().cmcg_format_dyn_line, C.byref(start), C.byref(end))


def lagrad_line(d: "Diag") -> str:
    return _fmt(lib().cmcg_format_lagrad_line, C.byref(d))


class Stars(C.Structure):
    """cmcg_stars: one cluster's host star arrays for cmcg_step_host."""
    _fields_ = [("N", C.c_long), ("cap", C.c_long)] + [(k, C.c_void_p) for k in ("r", "m", "vr", "vt", "E", "J", "id")]


STAR_KEYS = ("r", "m", "vr", "vt", "E", "J", "id")


class HostStars:
    """Every cluster's host star arrays, bound once for repeated steps in place
    (Context.step_host_inplace: cmcg_step_host with the same cmcg_stars array
    as input and output, so each step's star counts are the next step's
    input).  bufs[k] holds float64 arrays r, m, vr, vt, E, J and an int64 id,
    contiguous, of one length; ns[k] stars are taken from them."""

    def __init__(self, bufs, ns):
        self.bufs = list(bufs)  # the arrays must outlive the binding
        self.arr = (Stars * len(self.bufs))()
        for k, (b, n) in enumerate(zip(self.bufs, ns)):
            cap = len(b["r"])
            for x in STAR_KEYS:
                a = b[x]
                want = np.int64 if x == "id" else np.float64
                if a.dtype != want or not a.flags.c_contiguous or len(a) != cap:
                    raise ValueError(f"cluster {k}: array {x} must be contiguous {np.dtype(want)} of length {cap}")
            if not 0 <= n <= cap:
                raise ValueError(f"cluster {k}: {n} stars do not fit arrays of length {cap}")
            self.arr[k] = Stars(n, cap, *[b[x].ctypes.data for x in STAR_KEYS])

    def counts(self):
        return [int(s.N) for s in self.arr]


class CmcHdf5Info(C.Structure):
    """cmcg_cmc_hdf5_info: the attributes and table shapes of a CMC initial-conditions file."""
    _fields_ = [("nobj", C.c_long), ("nbinary", C.c_long), ("mclus", C.c_double), ("rvir", C.c_double),
                ("rtid", C.c_double), ("z", C.c_double), ("obj_rows", C.c_long), ("obj_cols", C.c_long),
                ("bin_rows", C.c_long), ("bin_cols", C.c_long)]


# the columns of the file's two tables, as cmc_read_hdf5_file (src/libs/fitslib.c:385-420) takes them
CMC_OBJ_COLUMNS = ("id", "k", "m", "Reff", "r", "vr", "vt", "binind")
CMC_BIN_COLUMNS = ("index", "id1", "k1", "m1", "Reff1", "id2", "k2", "m2", "Reff2", "a", "e")


class ICSpec(C.Structure):
    _fields_ = [("model", C.c_int), ("N", C.c_long), ("w0", C.c_double), ("imf", C.c_int),
                ("binary_fraction", C.c_double), ("seed", C.c_uint64)]


class ICOut(C.Structure):
    _fields_ = [("r", C.POINTER(C.c_double)), ("m", C.POINTER(C.c_double)), ("vr", C.POINTER(C.c_double)),
                ("vt", C.POINTER(C.c_double)), ("id", C.POINTER(C.c_int64)), ("rtid", C.c_double)]


class DropinHost(C.Structure):
    """cmcx_host of include/cmc_dropin.h."""
    _fields_ = [
        ("star", C.c_void_p), ("star_size", C.c_size_t),
        *[(f"off_{n}", C.c_long) for n in ("r", "vr", "vt", "m", "E", "J", "id", "rnew", "vrnew", "vtnew",
                                            "rOld", "X", "Y", "r_peri", "r_apo")],
        ("id_bytes", C.c_int),
        ("star_r", C.c_void_p), ("star_m", C.c_void_p), ("star_phi", C.c_void_p),
        ("N_STAR_DIM", C.c_long), ("N_MAX", C.c_void_p), ("N_MAX_NEW", C.c_void_p),
        *[(n, C.c_void_p) for n in ("Dt", "Mtotal", "Rtidal", "max_r", "Eescaped", "Jescaped", "TidalMassLoss",
                                     "Etidal", "Etot", "KE", "PE", "tcount")],
        ("sync_each", C.c_int),
    ]


ABORT_HANDLER = C.CFUNCTYPE(None, C.c_int, C.c_char_p)
DROPIN_PATH = os.path.join(_HERE, "_build", "libcmc_dropin.so")
DROPIN_FUNCS = {  # reference-named symbols: (restype, argtypes)
    "calc_timestep": (None, [C.c_void_p]), "dynamics_apply": (None, [C.c_double, C.c_void_p]),
    "energy_conservation1": (None, []), "energy_conservation2": (None, []),
    "new_orbits_calculate": (None, []), "get_positions": (C.c_double, []),
    "tidally_strip_stars": (None, []), "ComputeIntermediateEnergy": (None, []), "qsorts_new": (None, []),
    "post_sort_comm": (None, []), "potential_calculate": (C.c_long, []), "calc_potential_new": (None, []),
    "energy_conservation3": (None, []), "compute_energy_new": (None, []), "potential": (C.c_double, [C.c_double]),
}
_dropin = None


def dropin_lib() -> C.CDLL:
    """The reference-named drop-in library (include/cmc_dropin.h)."""
    global _dropin
    if _dropin is None:
        lib()
        if not os.path.exists(DROPIN_PATH):
            raise RuntimeError(f"{DROPIN_PATH} is missing: run cmc-cosmic_gb300/build.py")
        L = C.CDLL(DROPIN_PATH)
        for name, (res, args) in DROPIN_FUNCS.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        L.cmcx_default_host.argtypes = [C.POINTER(DropinHost)]
        L.cmcx_bind.argtypes = [C.POINTER(DropinHost), C.POINTER(Params)]
        L.cmcx_set_abort.argtypes = [ABORT_HANDLER]
        _dropin = L
    return _dropin


PLUMMER, KING = 0, 1
_lib = None


def build(force: bool = False) -> str:
    import importlib.util
    spec = importlib.util.spec_from_file_location("cmcg_build", os.path.join(_HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib() -> C.CDLL:
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run cmc-cosmic_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        vp, d, i, l = C.c_void_p, C.c_double, C.c_int, C.c_long
        L.cmcg_default_params.argtypes = [C.POINTER(Params)]
        L.cmcg_create.argtypes = [C.POINTER(vp), i, C.POINTER(l), C.POINTER(Params)]
        L.cmcg_destroy.argtypes = [vp]
        L.cmcg_load.argtypes = [vp, i, l, vp, vp, vp, vp, vp]
        for name in ["cmcg_initialize", "cmcg_begin_step", "cmcg_calc_timestep", "cmcg_new_orbits_calculate",
                     "cmcg_tidally_strip_stars", "cmcg_qsorts_new", "cmcg_calc_potential",
                     "cmcg_energy_conservation3", "cmcg_compute_energy", "cmcg_end_step", "cmcg_step",
                     "cmcg_synchronize"]:
            getattr(L, name).argtypes = [vp]
        L.cmcg_dynamics_apply.argtypes = [vp, d]
        L.cmcg_run.argtypes = [vp, i]
        L.cmcg_use_graph.argtypes = [vp, i]
        L.cmcg_profile.argtypes = [vp, i]
        L.cmcg_kernel_time.argtypes = [vp, C.c_char_p, C.POINTER(d), C.POINTER(l)]
        L.cmcg_potential.argtypes = [vp, i, d, C.POINTER(d)]
        L.cmcg_get_field.argtypes = [vp, i, C.c_char_p, vp, l]
        L.cmcg_get_field.restype = l
        L.cmcg_set_field.argtypes = [vp, i, C.c_char_p, vp, l]
        L.cmcg_set_field.restype = l
        L.cmcg_get_ids.argtypes = [vp, i, vp, l]
        L.cmcg_get_ids.restype = l
        L.cmcg_get_scalar.argtypes = [vp, i, C.c_char_p, C.POINTER(d)]
        L.cmcg_set_scalar.argtypes = [vp, i, C.c_char_p, d]
        L.cmcg_nstars.argtypes = [vp, i]
        L.cmcg_nstars.restype = l
        L.cmcg_last_error.argtypes = [vp, C.POINTER(i), C.POINTER(l)]
        L.cmcg_launch_count.argtypes = [vp]
        L.cmcg_launch_count.restype = l
        L.cmcg_stream.argtypes = [vp]
        L.cmcg_stream.restype = vp
        L.cmcg_ic_generate.argtypes = [C.POINTER(ICSpec), C.POINTER(ICOut)]
        L.cmcg_derive_seed.argtypes = [C.c_uint64, C.c_uint64]
        L.cmcg_derive_seed.restype = C.c_uint64
        L.cmcg_draw.argtypes = [C.c_uint64, l, i, C.c_int64, C.c_uint32, i]
        L.cmcg_draw.restype = d
        L.cmcg_sign_stages.argtypes = [vp, vp, vp, vp, d, vp, vp, l, vp]
        L.cmcg_trig_check.argtypes = [vp, l, vp, l, vp]
        L.cmcg_diagnostics.argtypes = [vp, i, vp, i, i, d, vp]
        L.cmcg_orbit_counters.argtypes = [vp, i]
        L.cmcg_format_dyn_line.argtypes = [vp, vp, vp, l]
        L.cmcg_format_dyn_line.restype = l
        L.cmcg_format_lagrad_line.argtypes = [vp, vp, l]
        L.cmcg_format_lagrad_line.restype = l
        L.cmcg_format_dyn_header.argtypes = [vp, l]
        L.cmcg_format_dyn_header.restype = l
        L.cmcg_format_lagrad_header.argtypes = [vp, i, vp, l]
        L.cmcg_format_lagrad_header.restype = l
        L.cmcg_sort_radii_noalloc.argtypes = [vp, l, vp, C.POINTER(l), vp]
        L.cmcg_put_stars.argtypes = [vp, i, l, vp, vp, vp, vp, vp, vp, vp]
        L.cmcg_get_stars.argtypes = [vp, i, l, vp, vp, vp, vp, vp, vp, vp]
        L.cmcg_get_stars.restype = l
        L.cmcg_set_learned.argtypes = [vp, i, d]
        L.cmcg_mlp_init.argtypes = [vp, C.c_uint64]
        L.cmcg_mlp_set_params.argtypes = [vp, vp]
        L.cmcg_mlp_get_params.argtypes = [vp, vp]
        L.cmcg_mlp_forward.argtypes = [vp, vp, l, vp, vp]
        L.cmcg_mlp_gradient.argtypes = [vp, vp, vp, vp, l, vp]
        L.cmcg_mlp_train.argtypes = [vp, vp, vp, vp, l, i, i, d, C.c_uint64, vp]
        L.cmcg_learned_samples.argtypes = [vp, i, vp, vp, vp, l]
        L.cmcg_learned_samples.restype = l
        L.cmcg_learned_stats.argtypes = [vp, vp]
        L.cmcg_autotune.argtypes = [vp, i, C.c_char_p, l]
        L.cmcg_step_host.argtypes = [vp, C.POINTER(Stars), C.POINTER(Stars)]
        L.cmcg_set_variant.argtypes = [vp, C.c_char_p, i]
        L.cmcg_get_variant.argtypes = [vp, C.c_char_p]
        _lib = L
    return _lib


_ic_lib = None


def ic_lib() -> C.CDLL:
    """libcmcic.so, the synthetic-cluster generator alone (no CUDA): models for
    the CPU oracle and baselines come from it without mapping the GPU library."""
    global _ic_lib
    if _ic_lib is None:
        if not os.path.exists(IC_LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("cmcg_build", os.path.join(_HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_ic()
        L = C.CDLL(IC_LIB_PATH)
        L.cmcg_ic_generate.argtypes = [C.POINTER(ICSpec), C.POINTER(ICOut)]
        L.cmcg_derive_seed.argtypes = [C.c_uint64, C.c_uint64]
        L.cmcg_read_cmc_hdf5.argtypes = [C.c_char_p, C.POINTER(CmcHdf5Info), C.c_void_p, C.c_long, C.c_void_p,
                                         C.c_long]
        L.cmcg_derive_seed.restype = C.c_uint64
        _ic_lib = L
    return _ic_lib


def header_symbols(path: str = HEADER) -> list[str]:
    """Function names the public header declares."""
    text = open(path).read()
    return sorted(set(re.findall(r"\b(cmcg_[a-z0-9_]+)\s*\(", text)))


def default_params(**kw) -> Params:
    p = Params()
    lib().cmcg_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def generate(model: int, N: int, seed: int, w0: float = 6.0, imf: int = 0, binary_fraction: float = 0.0):
    """Seeded synthetic cluster in N-body units; returns dict of arrays + rtid."""
    a = {k: np.zeros(N) for k in ("r", "m", "vr", "vt")}
    ids = np.zeros(N, np.int64)
    out = ICOut(*[a[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("r", "m", "vr", "vt")],
                ids.ctypes.data_as(C.POINTER(C.c_int64)), 0.0)
    rc = ic_lib().cmcg_ic_generate(C.byref(ICSpec(model, N, w0, imf, binary_fraction, seed)), C.byref(out))
    if rc:
        raise CmcError(rc, "cmcg_ic_generate")
    a["id"] = ids
    a["rtid"] = out.rtid
    return a


def derive_seed(master: int, index: int) -> int:
    return int(ic_lib().cmcg_derive_seed(master, index))


def read_cmc_hdf5(path: str) -> dict:
    """COSMIC's CMC initial-conditions file (cmcg_read_cmc_hdf5, read without
    the HDF5 library): {"info": the attributes and shapes, "obj": the object
    table, rows 0..NOBJ+1 (row 0 the central mass, the last the sentinel),
    columns CMC_OBJ_COLUMNS; "bin": the binary table, rows 0..NBINARY,
    columns CMC_BIN_COLUMNS}."""
    info = CmcHdf5Info()
    L = ic_lib()
    rc = L.cmcg_read_cmc_hdf5(os.fsencode(path), C.byref(info), None, 0, None, 0)
    if rc:
        raise CmcError(rc, "cmcg_read_cmc_hdf5")
    obj = np.zeros((info.obj_rows, info.obj_cols))
    binr = np.zeros((info.bin_rows, info.bin_cols))
    rc = L.cmcg_read_cmc_hdf5(os.fsencode(path), C.byref(info), obj.ctypes.data, info.obj_rows, binr.ctypes.data,
                              info.bin_rows)
    if rc:
        raise CmcError(rc, "cmcg_read_cmc_hdf5")
    return {"info": {k: getattr(info, k) for k, _ in CmcHdf5Info._fields_}, "obj": obj, "bin": binr}


def model_from_cmc_hdf5(path: str) -> dict:
    """A CMC initial-conditions file as a model for Context.load and the oracle:
    the NOBJ objects' r, m, vr, vt and id as the file holds them (N-body units,
    masses summing to 1 with the central mass), "rtid" the file's RTID,
    "cenma" row 0's mass (the central mass, cmc_fits.c:129-131), "binind" the
    objects' binary rows.  The plain Henon step treats a binary as a point
    mass of its object mass: with binary encounters off its cross-section is
    zero (cmc_dynamics.c:239-262)."""
    t = read_cmc_hdf5(path)
    obj, n = t["obj"], t["info"]["nobj"]
    col = {c: i for i, c in enumerate(CMC_OBJ_COLUMNS)}
    rows = obj[1:n + 1]
    return {"r": rows[:, col["r"]].copy(), "m": rows[:, col["m"]].copy(), "vr": rows[:, col["vr"]].copy(),
            "vt": rows[:, col["vt"]].copy(), "id": rows[:, col["id"]].astype(np.int64),
            "binind": rows[:, col["binind"]].astype(np.int64), "rtid": float(t["info"]["rtid"]),
            "cenma": float(obj[0, col["m"]])}


def draw(seed: int, tcount: int, site: int, star_id: int, n: int, word: int) -> float:
    return float(lib().cmcg_draw(seed, tcount, site, star_id, n, word))


ORBIT_COUNTERS = ("sign_f64", "sign_dd", "root_vr")


def orbit_counters(reset: bool = False) -> dict:
    """Rare-branch counts of the orbit phase on the current device since the
    last reset (cmcg_orbit_counters): probes decided in FP64, probes
    evaluated in double-double, apsides found by the root finder."""
    out = (C.c_ulonglong * 4)()
    rc = lib().cmcg_orbit_counters(out, int(reset))
    if rc:
        raise CmcError(rc, "cmcg_orbit_counters")
    return {k: int(out[i]) for i, k in enumerate(ORBIT_COUNTERS)}


def sign_stages(E, J, rj, mj, invN, rk, phik):
    """[n, 4] signs of function_q from the FP32, float-float, FP64 and
    double-double stages of the apsis sign test (0 = undecided)."""
    import numpy as np
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (E, J, rj, mj, rk, phik)]
    n = len(arrs[0])
    out = np.zeros((n, 4), np.int32)
    rc = lib().cmcg_sign_stages(*[a.ctypes.data for a in arrs[:4]], float(invN), arrs[4].ctypes.data,
                                arrs[5].ctypes.data, n, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"cmcg_sign_stages failed: {rc}")
    return out


def trig_check(w, beta):
    """The relaxation's FP32-pipe sines and cosines (cmcg_trig_check): [n, 2]
    (sin, cos) of 2 pi w 2^-32 for 32-bit draws w, and [nb, 2] of beta."""
    import numpy as np
    w = np.ascontiguousarray(w, dtype=np.uint32)
    b = np.ascontiguousarray(beta, dtype=np.float64)
    out = np.zeros(2 * (len(w) + len(b)))
    rc = lib().cmcg_trig_check(w.ctypes.data, len(w), b.ctypes.data, len(b), out.ctypes.data)
    if rc != 0:
        raise CmcError(rc, "cmcg_trig_check")
    return out[:2 * len(w)].reshape(-1, 2), out[2 * len(w):].reshape(-1, 2)


LEARN_OFF, LEARN_ON, LEARN_COLLECT = 0, 1, 2
MLP_NPARAM, MLP_NIN, MLP_NOUT, MLP_BINS = 6881, 8, 33, 32
LSTAT_NAMES = ("trials", "accepted", "failed", "stars", "plain_trials", "plain_stars")


class Context:
    """Clusters resident on the GPU; phases run all of them in one launch each."""

    def __init__(self, capacities, params):
        if isinstance(params, Params):
            params = [params] * len(capacities)
        self.n = len(capacities)
        caps = (C.c_long * self.n)(*capacities)
        ps = (Params * self.n)(*params)
        self._h = C.c_void_p()
        rc = lib().cmcg_create(C.byref(self._h), self.n, caps, ps)
        if rc:
            raise CmcError(rc, "cmcg_create")
        self.params = list(params)

    def close(self):
        if self._h:
            lib().cmcg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- data
    def load(self, cluster: int, r, m, vr, vt, ids=None):
        r, m, vr, vt = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, m, vr, vt))
        idp = None
        if ids is not None:
            ids = np.ascontiguousarray(ids, dtype=np.int64)
            idp = ids.ctypes.data
        self._check(lib().cmcg_load(self._h, cluster, len(r), r.ctypes.data, m.ctypes.data, vr.ctypes.data,
                                    vt.ctypes.data, idp), "cmcg_load")

    def _check(self, rc, where):
        if rc:
            raise CmcError(rc, where)

    def last_error(self):
        """(code, star index) of the first device error since the last call; (0, 0) if none."""
        c, idx = C.c_int(-1), C.c_long(0)
        rc = lib().cmcg_last_error(self._h, C.byref(c), C.byref(idx))
        return int(rc), int(idx.value)

    def check_device(self, where="device"):
        c, idx = C.c_int(-1), C.c_long(-1)
        rc = lib().cmcg_last_error(self._h, C.byref(c), C.byref(idx))
        if rc:
            raise CmcError(rc, f"{where} (cluster {c.value})", idx.value)

    def get(self, name: str, cluster: int = 0) -> np.ndarray:
        n = self.nstars(cluster) + 2
        out = np.zeros(max(n, 1))
        got = lib().cmcg_get_field(self._h, cluster, name.encode(), out.ctypes.data, len(out))
        if got < 0:
            raise KeyError(name)
        return out[:got].copy()

    def set(self, name: str, values, cluster: int = 0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if lib().cmcg_set_field(self._h, cluster, name.encode(), v.ctypes.data, len(v)) < 0:
            raise KeyError(name)

    def ids(self, cluster: int = 0) -> np.ndarray:
        n = self.nstars(cluster)
        out = np.zeros(max(n, 1), np.int64)
        got = lib().cmcg_get_ids(self._h, cluster, out.ctypes.data, len(out))
        return out[:got].copy()

    def scalar(self, name: str, cluster: int = 0) -> float:
        v = C.c_double()
        self._check(lib().cmcg_get_scalar(self._h, cluster, name.encode(), C.byref(v)), f"scalar {name}")
        return v.value

    def set_scalar(self, name: str, value: float, cluster: int = 0):
        self._check(lib().cmcg_set_scalar(self._h, cluster, name.encode(), float(value)), f"set_scalar {name}")

    def nstars(self, cluster: int = 0) -> int:
        return int(lib().cmcg_nstars(self._h, cluster))

    def potential(self, r: float, cluster: int = 0) -> float:
        v = C.c_double()
        self._check(lib().cmcg_potential(self._h, cluster, float(r), C.byref(v)), "potential")
        return v.value

    def diagnostics(self, cluster: int = 0, mass_pc=None, bh_include: int = 1, minimum_r: float = 0.0) -> "Diag":
        """The dyn.dat / lagrad.dat quantities of the cluster's current state (cmcg_diagnostics)."""
        pc = np.ascontiguousarray(MASS_PC if mass_pc is None else mass_pc, dtype=np.float64)
        d = Diag()
        self._check(lib().cmcg_diagnostics(self._h, cluster, pc.ctypes.data, len(pc), int(bh_include),
                                           float(minimum_r), C.byref(d)), "diagnostics")
        return d

    # -- phases (reference names)
    # -- learned proposal of the orbit sampler
    def set_learned(self, mode: int, kappa: float = 1.2):
        self._check(lib().cmcg_set_learned(self._h, mode, kappa), "cmcg_set_learned")

    def mlp_init(self, seed: int = 1):
        self._check(lib().cmcg_mlp_init(self._h, seed), "cmcg_mlp_init")

    def mlp_set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == MLP_NPARAM
        self._check(lib().cmcg_mlp_set_params(self._h, w.ctypes.data), "cmcg_mlp_set_params")

    def mlp_params(self) -> np.ndarray:
        w = np.zeros(MLP_NPARAM, np.float32)
        self._check(lib().cmcg_mlp_get_params(self._h, w.ctypes.data), "cmcg_mlp_get_params")
        return w

    def mlp_forward(self, feat):
        """(logits n x 33, proposal n x 32) of the network on feature rows n x 8."""
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NIN)
        n = feat.shape[0]
        z = np.zeros((n, MLP_NOUT), np.float32)
        p = np.zeros((n, MLP_BINS), np.float32)
        self._check(lib().cmcg_mlp_forward(self._h, feat.ctypes.data, n, z.ctypes.data, p.ctypes.data),
                    "cmcg_mlp_forward")
        return z, p

    def mlp_gradient(self, feat, bins, ntrial):
        """(mean gradient, (mean bin loss, mean trial loss)) over the records, no update."""
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NIN)
        bins = np.ascontiguousarray(bins, dtype=np.int32)
        ntrial = np.ascontiguousarray(ntrial, dtype=np.int32)
        g = np.zeros(MLP_NPARAM + 2, np.float32)
        self._check(lib().cmcg_mlp_gradient(self._h, feat.ctypes.data, bins.ctypes.data, ntrial.ctypes.data,
                                            feat.shape[0], g.ctypes.data), "cmcg_mlp_gradient")
        return g[:MLP_NPARAM], (float(g[MLP_NPARAM]), float(g[MLP_NPARAM + 1]))

    def mlp_train(self, feat, bins, ntrial, steps: int, batch: int = 8192, lr: float = 1e-3, seed: int = 1):
        """Adam steps on minibatches; returns the losses (steps x 2)."""
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NIN)
        bins = np.ascontiguousarray(bins, dtype=np.int32)
        ntrial = np.ascontiguousarray(ntrial, dtype=np.int32)
        loss = np.zeros((max(steps, 1), 2), np.float32)
        self._check(lib().cmcg_mlp_train(self._h, feat.ctypes.data, bins.ctypes.data, ntrial.ctypes.data,
                                         feat.shape[0], steps, batch, lr, seed, loss.ctypes.data), "cmcg_mlp_train")
        return loss[:steps]

    def learned_samples(self, cluster: int = 0):
        """(features n x 8, accepted X, trials) of the last step's sampled stars."""
        cap = self.nstars(cluster) + 2 + 128
        feat = np.zeros((cap, MLP_NIN), np.float32)
        X = np.zeros(cap)
        nt = np.zeros(cap, np.int32)
        n = lib().cmcg_learned_samples(self._h, cluster, feat.ctypes.data, X.ctypes.data, nt.ctypes.data, cap)
        if n < 0:
            raise CmcError(int(n), "cmcg_learned_samples")
        n = min(n, cap)
        return feat[:n], X[:n], nt[:n]

    def learned_stats(self) -> dict:
        out = np.zeros(8, np.uint64)
        self._check(lib().cmcg_learned_stats(self._h, out.ctypes.data), "cmcg_learned_stats")
        return {k: int(out[i]) for i, k in enumerate(LSTAT_NAMES)}

    # -- autotuner
    def autotune(self, steps: int = 2) -> str:
        """Time each launch variant over `steps` steps (real steps of the run), keep the fastest."""
        buf = C.create_string_buffer(1024)
        self._check(lib().cmcg_autotune(self._h, steps, buf, len(buf)), "cmcg_autotune")
        return buf.value.decode()

    def set_variant(self, name: str, v: int):
        self._check(lib().cmcg_set_variant(self._h, name.encode(), v), "cmcg_set_variant")

    def variant(self, name: str) -> int:
        v = lib().cmcg_get_variant(self._h, name.encode())
        if v < 0:
            raise KeyError(name)
        return v

    def initialize(self):
        self._check(lib().cmcg_initialize(self._h), "initialize")

    def begin_step(self):
        self._check(lib().cmcg_begin_step(self._h), "begin_step")

    def calc_timestep(self):
        self._check(lib().cmcg_calc_timestep(self._h), "calc_timestep")

    def dynamics_apply(self, dt: float = -1.0):
        self._check(lib().cmcg_dynamics_apply(self._h, dt), "dynamics_apply")

    def new_orbits_calculate(self):
        self._check(lib().cmcg_new_orbits_calculate(self._h), "new_orbits_calculate")

    def tidally_strip_stars(self):
        self._check(lib().cmcg_tidally_strip_stars(self._h), "tidally_strip_stars")

    def qsorts_new(self):
        self._check(lib().cmcg_qsorts_new(self._h), "qsorts_new")

    def calc_potential(self):
        self._check(lib().cmcg_calc_potential(self._h), "calc_potential")

    def energy_conservation3(self):
        self._check(lib().cmcg_energy_conservation3(self._h), "energy_conservation3")

    def compute_energy(self):
        self._check(lib().cmcg_compute_energy(self._h), "compute_energy")

    def end_step(self):
        self._check(lib().cmcg_end_step(self._h), "end_step")

    def step(self, n: int = 1):
        self._check(lib().cmcg_run(self._h, n), "run")

    def use_graph(self, on: bool = True):
        self._check(lib().cmcg_use_graph(self._h, 1 if on else 0), "use_graph")

    def profile(self, on: bool = True):
        self._check(lib().cmcg_profile(self._h, 1 if on else 0), "profile")

    def kernel_time(self, family: str):
        ms, n = C.c_double(), C.c_long()
        self._check(lib().cmcg_kernel_time(self._h, family.encode(), C.byref(ms), C.byref(n)), "kernel_time")
        return ms.value, n.value

    def synchronize(self):
        self._check(lib().cmcg_synchronize(self._h), "synchronize")

    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer (torch.cuda.ExternalStream takes it)."""
        return int(lib().cmcg_stream(self._h) or 0)

    def launch_count(self) -> int:
        return int(lib().cmcg_launch_count(self._h))

    def put_stars(self, cluster: int, n: int, bufs: dict):
        """Upload host star state (arrays r, m, vr, vt, E, J, id; m already x N_STAR)."""
        a = [bufs[k].ctypes.data for k in ("r", "m", "vr", "vt", "E", "J", "id")]
        self._check(lib().cmcg_put_stars(self._h, cluster, n, *a), "put_stars")

    def step_host_inplace(self, hs: HostStars):
        """One step on bound host arrays, in place (cmcg_step_host with in ==
        out); returns the star counts after it, which the binding keeps as the
        next step's input."""
        if len(hs.arr) != self.n:
            raise ValueError(f"binding holds {len(hs.arr)} clusters, the context {self.n}")
        self._check(lib().cmcg_step_host(self._h, hs.arr, hs.arr), "cmcg_step_host")
        return hs.counts()

    def step_host(self, ins, outs):
        """One step on host arrays: ins[k] = (n, bufs) per cluster, outs[k] = bufs
        (arrays r, m, vr, vt, E, J, id; cmcg_step_host).  Returns the star
        counts after the step."""
        keys = ("r", "m", "vr", "vt", "E", "J", "id")
        a = (Stars * self.n)()
        b = (Stars * self.n)()
        for k, ((n, bi), bo) in enumerate(zip(ins, outs)):
            a[k] = Stars(n, len(bi["r"]), *[bi[x].ctypes.data for x in keys])
            b[k] = Stars(0, len(bo["r"]), *[bo[x].ctypes.data for x in keys])
        self._check(lib().cmcg_step_host(self._h, a, b), "cmcg_step_host")
        return [int(b[k].N) for k in range(self.n)]

    def get_stars(self, cluster: int, bufs: dict) -> int:
        cap = len(bufs["r"])
        a = [bufs[k].ctypes.data for k in ("r", "m", "vr", "vt", "E", "J", "id")]
        n = lib().cmcg_get_stars(self._h, cluster, cap, *a)
        if n < 0:
            raise CmcError(int(n), "get_stars")
        return int(n)
