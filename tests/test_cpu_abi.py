"""The C-ABI libraries without a GPU: they load, export every function their
headers declare, and refuse to run (loudly) when no device is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
DECL = re.compile(r"^(?:void|int|long|double|uint64_t|cmcg_ctx\s*\*)\s*\**\s*([A-Za-z_]\w*)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(DECL.findall(text)))


def has_gpu(gpulib):
    n = C.c_int(0)
    try:
        cudart = C.CDLL("libcudart.so")
    except OSError:
        return False
    return cudart.cudaGetDeviceCount(C.byref(n)) == 0 and n.value > 0


def test_cmcgpu_exports_every_declared_function(gpulib):
    names = declared("cmcgpu.h")
    assert "cmcg_qsorts_new" in names and "cmcg_sort_radii_noalloc" in names and len(names) >= 36
    L = gpulib.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_dropin_exports_every_declared_function(gpulib):
    names = declared("cmc_dropin.h")
    # the reference's own names (include/cmc/cmc.h prototypes)
    for ref in ("qsorts_new", "post_sort_comm", "calc_potential_new", "potential_calculate", "dynamics_apply",
                "get_positions", "potential"):
        assert ref in names, ref
    L = gpulib.dropin_lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def struct_fields(header, name):
    """Member names of `typedef struct {...} name;` in declaration order."""
    text = open(os.path.join(INCLUDE, header)).read()
    body = re.search(r"typedef struct \{(.*?)\} " + name + ";", text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:unsigned\s+)?\w+\s+(.*)$", decl, re.S)
        fields += [n.strip(" *\n") for n in m.group(1).split(",")]
    return fields


def test_params_struct_matches_header(gpulib):
    """The ctypes mirrors list the headers' members in order."""
    assert struct_fields("cmcgpu.h", "cmcg_params") == [f for f, _ in gpulib.Params._fields_]


def test_dropin_host_struct_matches_header(gpulib):
    assert struct_fields("cmc_dropin.h", "cmcx_host") == [f for f, _ in gpulib.DropinHost._fields_]


def test_create_without_gpu_fails_loudly(gpulib):
    if has_gpu(gpulib):
        pytest.skip("a GPU is present")
    with pytest.raises(gpulib.CmcError) as e:
        gpulib.Context([1000], gpulib.default_params())
    assert e.value.code == -2  # CMCG_ERR_CUDA: no CPU fallback


def test_dropin_unbound_calls_report_through_the_abort_handler(gpulib):
    L = gpulib.dropin_lib()
    seen = []
    handler = gpulib.ABORT_HANDLER(lambda code, where: seen.append((code, where.decode())))
    L.cmcx_set_abort(handler)
    try:
        L.qsorts_new()
        L.calc_potential_new()
        assert L.potential(1.0) == 0.0
    finally:
        L.cmcx_set_abort(gpulib.ABORT_HANDLER())
    assert [c for c, _ in seen] == [-5, -5, -5]  # CMCG_ERR_STATE
    assert [w for _, w in seen] == ["qsorts_new", "potential_calculate", "potential"]


def test_dropin_bind_without_gpu_fails(gpulib):
    if has_gpu(gpulib):
        pytest.skip("a GPU is present")
    L = gpulib.dropin_lib()
    h = gpulib.DropinHost()
    L.cmcx_default_host(C.byref(h))
    star = np.zeros((102, 8))
    nmax = np.array([100], np.int64)
    h.star, h.star_size = star.ctypes.data, 64
    for i, f in enumerate(("r", "vr", "vt", "m", "E", "J", "id")):
        setattr(h, f"off_{f}", 8 * i)
    h.N_MAX = h.N_MAX_NEW = nmax.ctypes.data
    h.N_STAR_DIM = 102
    p = gpulib.default_params(N_STAR=100)
    assert L.cmcx_bind(C.byref(h), C.byref(p)) == -2


def test_ic_generator_is_seeded_and_sorted(gpulib):
    a = gpulib.generate(gpulib.KING, 5000, seed=7, imf=1)
    b = gpulib.generate(gpulib.KING, 5000, seed=7, imf=1)
    c = gpulib.generate(gpulib.KING, 5000, seed=8, imf=1)
    for k in ("r", "m", "vr", "vt"):
        assert np.array_equal(a[k], b[k])
    assert not np.array_equal(a["r"], c["r"])
    assert np.all(np.diff(a["r"]) >= 0)
    assert abs(a["m"].sum() - 1.0) < 1e-12


GLUE = r"""
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
typedef struct gsl_rng gsl_rng;
/* the reference's prototypes (include/cmc/cmc.h) as its host program sees them */
void dynamics_apply(double dt, gsl_rng *rng);
void calc_timestep(gsl_rng *rng);
void qsorts_new(void);
void post_sort_comm(void);
long potential_calculate(void);
void calc_potential_new(void);
double get_positions(void);
double potential(double r);
#define CMCX_NO_REFERENCE_PROTOTYPES
#include "cmc_dropin.h"

typedef struct { double r, vr, vt, m, E, J; long id; double rnew, pad[9]; int se; } star_t;
static star_t star[1002];
static double star_r[1002], star_m[1002], star_phi[1002];
static long N_MAX = 1000, N_MAX_NEW = 1000;
static int seen;
static void on_error(int code, const char *where) { (void)where; seen = code; }

int main(void) {
    cmcx_host h;
    cmcx_default_host(&h);
    for (long i = 1; i <= 1000; i++) { star[i].r = i * 1e-3; star[i].m = 1.0; star[i].vt = 0.5; star[i].id = i; }
    h.star = star; h.star_size = sizeof(star_t);
    h.off_r = offsetof(star_t, r); h.off_vr = offsetof(star_t, vr); h.off_vt = offsetof(star_t, vt);
    h.off_m = offsetof(star_t, m); h.off_E = offsetof(star_t, E); h.off_J = offsetof(star_t, J);
    h.off_id = offsetof(star_t, id); h.off_rnew = offsetof(star_t, rnew); h.id_bytes = sizeof(star[0].id);
    h.star_r = star_r; h.star_m = star_m; h.star_phi = star_phi; h.N_STAR_DIM = 1002;
    h.N_MAX = &N_MAX; h.N_MAX_NEW = &N_MAX_NEW;
    cmcg_params p;
    cmcg_default_params(&p);
    p.N_STAR = 1000;
    cmcx_set_abort(on_error);
    int rc = cmcx_bind(&h, &p);
    if (rc == 0) {              /* a GPU is present: one potential through the reference's name */
        calc_potential_new();
        rc = seen || !(star_phi[1] < 0.0) || potential(0.5) >= 0.0;
        cmcx_unbind();
        printf("bound %d\n", rc);
        return rc;
    }
    printf("no device %d\n", rc);
    return rc == CMCG_ERR_CUDA ? 0 : 1;
}
"""


def test_c_host_with_reference_prototypes_links_and_runs(gpulib, tmp_path):
    """A C program declaring the reference's prototypes (gsl_rng *) and its
    own star_t compiles against cmc_dropin.h, links against the drop-in, and
    runs: without a GPU the bind reports CMCG_ERR_CUDA, with one it computes
    a potential through calc_potential_new()."""
    import subprocess
    gpulib.dropin_lib()
    src = tmp_path / "glue.c"
    src.write_text(GLUE)
    exe = tmp_path / "glue"
    build = os.path.join(ROOT, "cmc-cosmic_gb300", "_build")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I" + INCLUDE, str(src), "-o", str(exe), "-L" + build,
                    "-lcmc_dropin", "-lcmcgpu", "-Wl,-rpath," + build], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr


def test_host_stars_binding_checks_its_arrays(gpulib):
    """HostStars (the in-place host-exchange binding) refuses arrays the C side
    would misread: wrong dtype, non-contiguous, unequal lengths, too many stars.
    No GPU is touched."""
    import numpy as np

    def bufs(n):
        b = {k: np.zeros(n) for k in ("r", "m", "vr", "vt", "E", "J")}
        b["id"] = np.zeros(n, np.int64)
        return b

    hs = gpulib.HostStars([bufs(100), bufs(50)], [90, 50])
    assert hs.counts() == [90, 50]
    bad = bufs(100)
    bad["id"] = np.zeros(100)  # float64 ids
    with pytest.raises(ValueError):
        gpulib.HostStars([bad], [10])
    bad = bufs(100)
    bad["E"] = np.zeros(200)[::2]  # strided
    with pytest.raises(ValueError):
        gpulib.HostStars([bad], [10])
    bad = bufs(100)
    bad["J"] = np.zeros(99)
    with pytest.raises(ValueError):
        gpulib.HostStars([bad], [10])
    with pytest.raises(ValueError):
        gpulib.HostStars([bufs(100)], [101])
