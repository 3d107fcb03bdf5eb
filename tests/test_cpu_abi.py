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
