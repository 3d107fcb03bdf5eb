"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

The oracle (cmc_oracle.c) restates the reference's single-rank Henon step in C
and is the parity checker for the GPU kernels.  Only the tests, the smoke
check and bench.py's CPU-baseline leg use it.

``build()`` compiles it into oracle/_build.  ``build_ref()`` runs the recipe
oracle/ref.mk where the reference tree is present: it compiles the
reference's own Henon-step TUs in place against single-rank MPI / GSL / HDF5
shims (oracle/refshim) into oracle/_ref/libcmcref.so, and the reference's
taus113 generator into oracle/_ref/libtaus113ref.so.  ``RefOracle`` drives
libcmcref.so with the same interface as ``Oracle``, so that the restatement
is pinned to the reference's own code phase by phase.  Both build folders
stay outside version control.  The reference tree is $CMC_REFERENCE_ROOT, or
the recipe's default.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcmcoracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_TAUS = os.path.join(REF_DIR, "libtaus113ref.so")
REF_LIB = os.path.join(REF_DIR, "libcmcref.so")
REF_MK = os.path.join(HERE, "ref.mk")

DRAW_COUNTER, DRAW_TAUS113 = 0, 1
SITE_Y, SITE_PENC, SITE_PSI, SITE_TRIAL, SITE_SIGN = 1, 2, 3, 4, 5
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11"]


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "cmc_oracle.c")
    hdr = os.path.join(HERE, "cmc_oracle.h")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.check_call(["gcc", *CFLAGS, "-shared", "-o", LIB, src, "-lm"])
    return LIB


def reference_root() -> str | None:
    """The reference tree: $CMC_REFERENCE_ROOT, else the recipe's default;
    None when it is not there (as on a machine without the reference)."""
    root = os.environ.get("CMC_REFERENCE_ROOT")
    if not root:
        res = subprocess.run(["make", "-s", "-f", REF_MK, "print-root"], capture_output=True, text=True)
        root = res.stdout.strip()
    if root and os.path.exists(os.path.join(root, "src", "cmc", "cmc_utils.c")):
        return root
    return None


def build_ref() -> str | None:
    """Build oracle/_ref (libcmcref.so, libtaus113ref.so) with oracle/ref.mk;
    returns the reference-step library, or None when the reference tree is
    absent."""
    root = reference_root()
    if root is None:
        return None
    jobs = str(min(8, os.cpu_count() or 2))
    subprocess.check_call(["make", "-s", "-j", jobs, "-f", REF_MK, f"REFERENCE_ROOT={root}", "all"],
                          stdout=subprocess.DEVNULL)
    return REF_LIB


class OParams(C.Structure):
    _fields_ = [
        ("N_STAR", C.c_long), ("AVEKERNEL", C.c_long), ("GAMMA", C.c_double), ("THETASEMAX", C.c_double),
        ("PERTURB", C.c_int), ("RELAXATION", C.c_int), ("TIDALLY_STRIP_STARS", C.c_int),
        ("TIDAL_TREATMENT", C.c_int), ("orbit_r", C.c_double), ("cenma_m", C.c_double),
        ("apsides_max_iter", C.c_long), ("apsides_precision", C.c_double),
        ("apsides_convergence", C.c_double), ("n_try", C.c_long), ("seed", C.c_uint64), ("draw_mode", C.c_int),
    ]


OCMC_MASS_PC_MAX = 64


class ODiag(C.Structure):
    """ocmc_diag (cmc_oracle.h)."""
    _fields_ = ([("nave", C.c_long), ("rh", C.c_double)]
                + [(n, C.c_double) for n in ("rho", "v_rms", "rc", "rc_nb", "m_ave", "n", "rc_spitzer",
                                            "N_core", "N_core_nb", "Trc")]
                + [("n_pc", C.c_int)]
                + [(n, C.c_double * OCMC_MASS_PC_MAX) for n in ("mass_r", "ave_mass_r", "no_star_r", "densities_r",
                                                                "ke_rad_r", "ke_tan_r", "v2_rad_r", "v2_tan_r")])


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.ocmc_default_params.argtypes = [C.POINTER(OParams)]
        L.ocmc_create.argtypes = [C.POINTER(OParams), C.c_long, vp, vp, vp, vp, vp]
        L.ocmc_create.restype = vp
        L.ocmc_destroy.argtypes = [vp]
        for n in ["ocmc_initialize", "ocmc_begin_step", "ocmc_calc_timestep", "ocmc_energy_conservation1",
                  "ocmc_new_orbits_calculate", "ocmc_energy_conservation2", "ocmc_tidally_strip_stars",
                  "ocmc_compute_intermediate_energy", "ocmc_qsorts_new", "ocmc_calc_potential",
                  "ocmc_energy_conservation3", "ocmc_compute_energy", "ocmc_end_step", "ocmc_step",
                  "ocmc_last_error", "ocmc_nstars"]:
            getattr(L, n).argtypes = [vp]
        L.ocmc_nstars.restype = C.c_long
        L.ocmc_dynamics_apply.argtypes = [vp, C.c_double]
        L.ocmc_potential.argtypes = [vp, C.c_double]
        L.ocmc_potential.restype = C.c_double
        L.ocmc_get_field.argtypes = [vp, C.c_char_p, vp, C.c_long]
        L.ocmc_get_field.restype = C.c_long
        L.ocmc_set_field.argtypes = [vp, C.c_char_p, vp, C.c_long]
        L.ocmc_set_field.restype = C.c_long
        L.ocmc_get_ids.argtypes = [vp, vp, C.c_long]
        L.ocmc_get_ids.restype = C.c_long
        L.ocmc_get_scalar.argtypes = [vp, C.c_char_p]
        L.ocmc_get_scalar.restype = C.c_double
        L.ocmc_set_scalar.argtypes = [vp, C.c_char_p, C.c_double]
        L.ocmc_last_error_index.argtypes = [vp]
        L.ocmc_last_error_index.restype = C.c_long
        L.ocmc_draw.argtypes = [vp, C.c_int, C.c_int64, C.c_uint32, C.c_int]
        L.ocmc_draw.restype = C.c_double
        L.ocmc_philox4x32_10.argtypes = [vp, vp, vp]
        L.ocmc_taus113_seed.argtypes = [vp, C.c_ulong]
        L.ocmc_taus113_next.argtypes = [vp]
        L.ocmc_taus113_next.restype = C.c_uint32
        L.ocmc_diagnostics.argtypes = [vp, vp, C.c_int, C.c_int, C.c_double, C.POINTER(ODiag)]
        _lib = L
    return _lib


def default_params(**kw) -> OParams:
    p = OParams()
    lib().ocmc_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class OracleError(RuntimeError):
    def __init__(self, code, where, index):
        self.code, self.index = code, index
        super().__init__(f"oracle {where}: error {code} at {index}")


class Oracle:
    """One cluster stepped by the CPU restatement of the reference."""

    def __init__(self, ic: dict, params: OParams):
        r, m, vr, vt = (np.ascontiguousarray(ic[k], dtype=np.float64) for k in ("r", "m", "vr", "vt"))
        ids = np.ascontiguousarray(ic.get("id", np.arange(1, len(r) + 1)), dtype=np.int64)
        self.params = params
        self._h = lib().ocmc_create(C.byref(params), len(r), r.ctypes.data, m.ctypes.data, vr.ctypes.data,
                                    vt.ctypes.data, ids.ctypes.data)
        if not self._h:
            raise ValueError("ocmc_create failed")

    def close(self):
        if self._h:
            lib().ocmc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        rc = getattr(lib(), name)(self._h, *args)
        if rc:
            raise OracleError(rc, name, lib().ocmc_last_error_index(self._h))

    def __getattr__(self, item):
        fn = "ocmc_" + item
        if item.startswith("_") or not hasattr(lib(), fn):
            raise AttributeError(item)
        return lambda *a: self._call(fn, *a)

    def get(self, name: str) -> np.ndarray:
        n = lib().ocmc_nstars(self._h) + 2
        out = np.zeros(n)
        got = lib().ocmc_get_field(self._h, name.encode(), out.ctypes.data, n)
        if got < 0:
            raise KeyError(name)
        return out[:got].copy()

    def set(self, name: str, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if lib().ocmc_set_field(self._h, name.encode(), v.ctypes.data, len(v)) < 0:
            raise KeyError(name)

    def ids(self) -> np.ndarray:
        n = lib().ocmc_nstars(self._h)
        out = np.zeros(max(n, 1), np.int64)
        got = lib().ocmc_get_ids(self._h, out.ctypes.data, len(out))
        return out[:got].copy()

    def scalar(self, name: str) -> float:
        return float(lib().ocmc_get_scalar(self._h, name.encode()))

    def set_scalar(self, name: str, v: float):
        if lib().ocmc_set_scalar(self._h, name.encode(), float(v)):
            raise KeyError(name)

    def potential(self, r: float) -> float:
        return float(lib().ocmc_potential(self._h, float(r)))

    def diagnostics(self, mass_pc, bh_include: int = 1, minimum_r: float = 0.0) -> dict:
        """central_calculate, clusdyn_calculate and comp_mass_percent, sequentially."""
        pc = np.ascontiguousarray(mass_pc, dtype=np.float64)
        d = ODiag()
        if lib().ocmc_diagnostics(self._h, pc.ctypes.data, len(pc), int(bh_include), float(minimum_r),
                                  C.byref(d)):
            raise OracleError(lib().ocmc_last_error(self._h), "diagnostics", lib().ocmc_last_error_index(self._h))
        n = len(pc)
        out = {k: getattr(d, k) for k in ("nave", "rh", "rho", "v_rms", "rc", "rc_nb", "m_ave", "n", "rc_spitzer",
                                          "N_core", "N_core_nb", "Trc")}
        for k in ("mass_r", "ave_mass_r", "no_star_r", "densities_r", "ke_rad_r", "ke_tan_r", "v2_rad_r",
                  "v2_tan_r"):
            out[k] = np.array(getattr(d, k)[:n])
        return out

    def nstars(self) -> int:
        return int(lib().ocmc_nstars(self._h))

    def draw(self, site, star_id, n, word):
        return float(lib().ocmc_draw(self._h, site, star_id, n, word))


def ref_lib() -> C.CDLL:
    """A private copy of oracle/_ref/libcmcref.so, the reference's own step
    (see build_ref).  The reference keeps its whole state in globals and
    expects one run per process, so each caller gets its own copy of the
    library, loaded from a temporary file: its globals start zeroed, as in a
    fresh process, and no two instances share them."""
    import shutil
    import tempfile

    path = build_ref()
    if path is None:
        raise RuntimeError("the reference tree is not present: libcmcref.so cannot be built")
    fd, tmp = tempfile.mkstemp(prefix="cmcref_", suffix=".so")
    os.close(fd)
    try:
        shutil.copyfile(path, tmp)
        L = C.CDLL(tmp, mode=getattr(os, "RTLD_LOCAL", 0))
    finally:
        os.unlink(tmp)
    vp = C.c_void_p
    L.cmcref_create.argtypes = [C.POINTER(OParams), C.c_long, vp, vp, vp, vp, vp]
    for n in ["cmcref_initialize", "cmcref_begin_step", "cmcref_calc_timestep", "cmcref_energy_conservation1",
              "cmcref_new_orbits_calculate", "cmcref_energy_conservation2", "cmcref_tidally_strip_stars",
              "cmcref_compute_intermediate_energy", "cmcref_qsorts_new", "cmcref_calc_potential",
              "cmcref_energy_conservation3", "cmcref_compute_energy", "cmcref_end_step", "cmcref_step",
              "cmcref_last_error", "cmcref_sizeof_star"]:
        getattr(L, n).argtypes = []
    L.cmcref_nstars.restype = C.c_long
    L.cmcref_dynamics_apply.argtypes = [C.c_double]
    L.cmcref_potential.argtypes = [C.c_double]
    L.cmcref_potential.restype = C.c_double
    L.cmcref_get_field.argtypes = [C.c_char_p, vp, C.c_long]
    L.cmcref_get_field.restype = C.c_long
    L.cmcref_set_field.argtypes = [C.c_char_p, vp, C.c_long]
    L.cmcref_set_field.restype = C.c_long
    L.cmcref_get_ids.argtypes = [vp, C.c_long]
    L.cmcref_get_ids.restype = C.c_long
    L.cmcref_get_scalar.argtypes = [C.c_char_p]
    L.cmcref_get_scalar.restype = C.c_double
    L.cmcref_set_scalar.argtypes = [C.c_char_p, C.c_double]
    L.cmcref_last_error_what.restype = C.c_char_p
    return L


class RefOracle:
    """One cluster stepped by the reference's own code (libcmcref.so), with the
    same interface as Oracle; each instance has its own copy of the library."""

    def __init__(self, ic: dict, params: OParams):
        r, m, vr, vt = (np.ascontiguousarray(ic[k], dtype=np.float64) for k in ("r", "m", "vr", "vt"))
        ids = np.ascontiguousarray(ic.get("id", np.arange(1, len(r) + 1)), dtype=np.int64)
        self.params = params
        self._L = L = ref_lib()
        rc = L.cmcref_create(C.byref(params), len(r), r.ctypes.data, m.ctypes.data, vr.ctypes.data,
                             vt.ctypes.data, ids.ctypes.data)
        if rc:
            raise OracleError(rc, "cmcref_create (" + L.cmcref_last_error_what().decode() + ")", -1)
        self._open = True

    def close(self):
        if self._open:
            self._L.cmcref_destroy()
            self._open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        L = self._L
        rc = getattr(L, name)(*args)
        if rc:
            raise OracleError(rc, name + " (" + L.cmcref_last_error_what().decode() + ")", -1)

    def __getattr__(self, item):
        fn = "cmcref_" + item
        if item.startswith("_") or not hasattr(self._L, fn):
            raise AttributeError(item)
        return lambda *a: self._call(fn, *a)

    def get(self, name: str) -> np.ndarray:
        n = self._L.cmcref_nstars() + 2
        out = np.zeros(max(n, 2))
        got = self._L.cmcref_get_field(name.encode(), out.ctypes.data, len(out))
        if got < 0:
            raise KeyError(name)
        return out[:got].copy()

    def set(self, name: str, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if self._L.cmcref_set_field(name.encode(), v.ctypes.data, len(v)) < 0:
            raise KeyError(name)

    def ids(self) -> np.ndarray:
        n = self._L.cmcref_nstars()
        out = np.zeros(max(n, 1), np.int64)
        got = self._L.cmcref_get_ids(out.ctypes.data, len(out))
        return out[:got].copy()

    def scalar(self, name: str) -> float:
        return float(self._L.cmcref_get_scalar(name.encode()))

    def set_scalar(self, name: str, v: float):
        if self._L.cmcref_set_scalar(name.encode(), float(v)):
            raise KeyError(name)

    def potential(self, r: float) -> float:
        return float(self._L.cmcref_potential(float(r)))

    def nstars(self) -> int:
        return int(self._L.cmcref_nstars())


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().ocmc_philox4x32_10(c, k, o)
    return list(o)


def taus113_stream(seed: int, n: int) -> np.ndarray:
    z = (C.c_uint32 * 4)()
    lib().ocmc_taus113_seed(z, seed)
    return np.array([lib().ocmc_taus113_next(z) for _ in range(n)], dtype=np.uint64)
