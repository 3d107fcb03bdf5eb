"""The drop-in boundary against the reference's own headers and objects.

cmc-cosmic_gb300/csrc/cmc_gpu_glue.c is the file a maintainer adds to the
reference's build.  Here it is compiled against the reference's include/cmc
headers (with the single-rank MPI / GSL / HDF5 shims of oracle/refshim
standing in for the libraries this image lacks), which checks every
offsetof(star_t, ...) and every host pointer the binding takes.  Then the
reference's hot-path TUs are compiled with the definitions libcmc_dropin.so
replaces renamed away (with -D<name>=reference_<name>, the maintainer's route), and linked
with the glue and a main that references every replaced function: the link
must succeed with each of them resolved from libcmc_dropin.so.  Needs the
reference tree; nothing runs on a GPU."""
import os
import subprocess

import pytest

import cmcgpu
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.reference_root()
pytestmark = pytest.mark.skipif(REF is None, reason="reference tree not present")

# the reference's functions libcmc_dropin.so defines (include/cmc_dropin.h)
REPLACED = ["calc_timestep", "dynamics_apply", "energy_conservation1", "energy_conservation2",
            "new_orbits_calculate", "get_positions", "tidally_strip_stars", "ComputeIntermediateEnergy",
            "qsorts_new", "post_sort_comm", "potential_calculate", "calc_potential_new",
            "energy_conservation3", "compute_energy_new", "potential"]
TUS = ["cmc_utils", "cmc_dynamics", "cmc_dynamics_helper", "cmc_evolution_thr", "cmc_orbit", "cmc_nr", "cmc_sort",
       "cmc_fits", "cmc_mpi"]


def _flags():
    return ["-std=gnu11", "-fcommon", "-DEXPERIMENTAL", "-w", "-I", os.path.join(ROOT, "oracle", "refshim"),
            "-I", os.path.join(REF, "include", "cmc"), "-I", os.path.join(REF, "include", "common"),
            "-I", os.path.join(REF, "include"), "-I", os.path.join(ROOT, "include")]


def _cc(args):
    res = subprocess.run(["gcc", *args], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    return res


def test_glue_compiles_against_the_reference_headers(tmp_path):
    glue = os.path.join(ROOT, "cmc-cosmic_gb300", "csrc", "cmc_gpu_glue.c")
    res = _cc([*_flags(), "-Wall", "-Werror=incompatible-pointer-types", "-Werror=int-conversion",
               "-Werror=implicit-function-declaration", "-c", glue, "-o", str(tmp_path / "glue.o")])
    assert "warning" not in res.stderr


def test_reference_objects_link_against_the_dropin_library(tmp_path):
    cmcgpu.build()
    build = os.path.join(ROOT, "cmc-cosmic_gb300", "_build")
    renames = [f"-D{name}=reference_{name}" for name in REPLACED]
    objs = []
    for tu in TUS:
        o = str(tmp_path / f"{tu}.o")
        _cc([*_flags(), *renames, "-c", os.path.join(REF, "src", "cmc", f"{tu}.c"), "-o", o])
        objs.append(o)
    for src, inc in ((os.path.join(REF, "src", "fewbody-0.24", "fewbody_utils.c"),
                      ["-I", os.path.join(REF, "include", "fewbody-0.24")]),
                     (os.path.join(REF, "src", "libs", "taus113-v2.c"), [])):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        _cc([*_flags(), *inc, "-c", src, "-o", o])
        objs.append(o)
    for src in ("refshim.c", "refstubs.c"):
        o = str(tmp_path / (src + ".o"))
        _cc([*_flags(), "-c", os.path.join(ROOT, "oracle", "refshim", src), "-o", o])
        objs.append(o)
    glue = str(tmp_path / "glue.o")
    _cc([*_flags(), "-c", os.path.join(ROOT, "cmc-cosmic_gb300", "csrc", "cmc_gpu_glue.c"), "-o", glue])
    main_c = tmp_path / "main.c"
    main_c.write_text(
        '#include <stdio.h>\n#include <stdlib.h>\n#include "cmc.h"\n#include "cmc_vars.h"\n'
        "void cmc_gpu_bind(void);\n"
        "void cmcref_exit(int c) { exit(c); }\n"
        'void cmcref_unreachable(const char *w) { fprintf(stderr, "%s\\n", w); exit(1); }\n'
        "int main(int argc, char **argv) {\n"
        "    /* every replaced function, by its reference prototype */\n"
        "    void (*f0)(gsl_rng *) = calc_timestep; void (*f1)(double, gsl_rng *) = dynamics_apply;\n"
        "    void (*f2)(void) = energy_conservation1; void (*f3)(void) = energy_conservation2;\n"
        "    void (*f4)(void) = new_orbits_calculate; double (*f5)(void) = get_positions;\n"
        "    void (*f6)(void) = tidally_strip_stars; void (*f7)(void) = ComputeIntermediateEnergy;\n"
        "    void (*f8)(void) = qsorts_new; void (*f9)(void) = post_sort_comm;\n"
        "    long (*f10)(void) = potential_calculate; void (*f11)(void) = calc_potential_new;\n"
        "    void (*f12)(void) = energy_conservation3; void (*f13)(void) = compute_energy_new;\n"
        "    double (*f14)(double) = potential;\n"
        "    void *all[] = {f0, f1, f2, f3, f4, f5, f6, f7, f8, f9, f10, f11, f12, f13, f14};\n"
        "    if (argc > 99) cmc_gpu_bind();\n"
        "    return all[argc % 15] == NULL;\n}\n")
    mo = str(tmp_path / "main.o")
    _cc([*_flags(), "-c", str(main_c), "-o", mo])
    exe = str(tmp_path / "cmc_dropin_linked")
    _cc(["-o", exe, mo, glue, *objs, "-L" + build, "-lcmc_dropin", "-lcmcgpu", "-Wl,-rpath," + build, "-lm", "-lz"])
    # the replaced functions come from the shared library, not from the objects
    undef = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout.split()
    for name in REPLACED:
        assert name in undef, name
    defined = subprocess.run(["nm", "--defined-only", exe], capture_output=True, text=True).stdout.split()
    for name in REPLACED:
        assert "reference_" + name in defined, name
