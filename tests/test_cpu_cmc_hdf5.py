"""COSMIC's CMC initial-conditions file, read without the HDF5 library.

cmcg_read_cmc_hdf5 (cmc-cosmic_gb300/csrc/cmcg_h5.c) replaces the
reference's cmc_read_hdf5_file (src/libs/fitslib.c:209-455).  The
reference's own CI input, ci/input.hdf5 (written by
ci/make_initial_conditions.py: COSMIC's sampler, 10,000 objects, binary
fraction 0.2, metallicity 0.014, r_max 100, a Plummer profile), pins it:
the attributes and table shapes the reference's loader relies on, the
sentinel rows cmc_fits.c:63-136 expects, and the consistency of the object
and binary tables.  Then the reference's compiled step (oracle/ref.mk) and
the oracle step that model through the main loop's phases bit for bit.
Needs the reference tree; skips elsewhere.  Malformed files are refused."""
import os
import shutil

import numpy as np
import pytest

import cmcgpu
import oracle

REF = oracle.reference_root()
CI_INPUT = os.path.join(REF, "ci", "input.hdf5") if REF else None
pytestmark = pytest.mark.skipif(CI_INPUT is None or not os.path.exists(CI_INPUT),
                                reason="reference tree not present")

SF_INFINITY = 1e40  # include/cmc/cmc.h: the outer sentinel radius


def _col(name):
    return cmcgpu.CMC_OBJ_COLUMNS.index(name)


def _bcol(name):
    return cmcgpu.CMC_BIN_COLUMNS.index(name)


def test_reads_the_reference_ci_input():
    t = cmcgpu.read_cmc_hdf5(CI_INPUT)
    info, obj, b = t["info"], t["obj"], t["bin"]
    n, nb = info["nobj"], info["nbinary"]
    # the generating script's parameters
    assert n == 10000
    assert info["z"] == 0.014
    assert 1800 <= nb <= 2200  # binary fraction 0.2
    # the shapes cmc_read_hdf5_file and load_fits_file_data index
    assert obj.shape == (n + 2, 8) and b.shape == (nb + 1, 11)
    assert (info["obj_rows"], info["obj_cols"], info["bin_rows"], info["bin_cols"]) == (n + 2, 8, nb + 1, 11)
    # rows 0 and N+1: the central mass and the outer sentinel
    assert obj[n + 1, _col("r")] == SF_INFINITY
    assert 0.0 <= obj[0, _col("r")] < 1e-300
    rows = obj[1:n + 1]
    r, m = rows[:, _col("r")], rows[:, _col("m")]
    assert np.all(r > 0) and np.all(np.diff(r) >= 0) and r.max() <= 100.0  # sorted, within r_max
    assert np.all(m > 0)
    assert abs(m.sum() + obj[0, _col("m")] - 1.0) <= 1e-12  # N-body mass units
    ids = rows[:, _col("id")]
    assert np.array_equal(np.sort(ids), np.arange(1, n + 1))
    # every binary is one object's: indices a permutation, id1 the object's id, m = m1 + m2
    bi = rows[:, _col("binind")].astype(np.int64)
    sel = bi > 0
    assert np.array_equal(np.sort(bi[sel]), np.arange(1, nb + 1))
    assert np.array_equal(b[1:, _bcol("index")], np.arange(1, nb + 1))
    assert np.array_equal(b[bi[sel], _bcol("id1")], ids[sel])
    m12 = b[bi[sel], _bcol("m1")] + b[bi[sel], _bcol("m2")]
    assert np.max(np.abs(m[sel] - m12) / m[sel]) <= 4e-16
    assert np.all(b[1:, _bcol("e")] >= 0) and np.all(b[1:, _bcol("e")] < 1) and np.all(b[1:, _bcol("a")] > 0)


def test_model_from_the_ci_input():
    ic = cmcgpu.model_from_cmc_hdf5(CI_INPUT)
    t = cmcgpu.read_cmc_hdf5(CI_INPUT)
    n = t["info"]["nobj"]
    assert len(ic["r"]) == n and ic["rtid"] == t["info"]["rtid"] and ic["cenma"] == t["obj"][0, _col("m")]
    for k in ("r", "m", "vr", "vt"):
        assert np.array_equal(ic[k], t["obj"][1:n + 1, _col(k)]), k


def test_reference_and_oracle_step_the_ci_input_bit_identically():
    """The reference's CI model through the reference's compiled step and the
    oracle, three steps phase by phase (every per-star field, global array and
    scalar equal after every phase).  Binaries step as point masses of their
    object mass: with binary encounters off (the plain configuration) their
    cross-section is zero and the encounter draw is taken as for singles
    (cmc_dynamics.c:239-262, 406)."""
    from test_cpu_refpin import _run_phases

    if oracle.build_ref() is None:
        pytest.skip("reference tree not present")
    oracle.build()
    ic = cmcgpu.model_from_cmc_hdf5(CI_INPUT)
    assert ic["cenma"] == 0.0  # the sampler puts no central mass in row 0
    # RTID = 1e6 N-body lengths: no star is ever stripped
    etot = _run_phases(ic, steps=3)
    assert all(a == b for a, b in etot)


def test_refuses_what_it_does_not_read(tmp_path):
    with pytest.raises(cmcgpu.CmcError) as e:
        cmcgpu.read_cmc_hdf5(str(tmp_path / "absent.hdf5"))
    assert e.value.code == cmcgpu.CMCG_ERR_IO
    data = open(CI_INPUT, "rb").read()
    cases = {
        "truncated": data[:4096],                       # structures point past the end
        "not_hdf5": b"\0" * 4096,                        # no signature
        "superblock_v2": data[:8] + b"\x02" + data[9:],  # a superblock version it does not read
    }
    for name, blob in cases.items():
        p = tmp_path / f"{name}.hdf5"
        p.write_bytes(blob)
        with pytest.raises(cmcgpu.CmcError) as e:
            cmcgpu.read_cmc_hdf5(str(p))
        assert e.value.code == cmcgpu.CMCG_ERR_FORMAT, name
    # an intact copy still reads
    shutil.copy(CI_INPUT, tmp_path / "copy.hdf5")
    assert cmcgpu.read_cmc_hdf5(str(tmp_path / "copy.hdf5"))["info"]["nobj"] == 10000
