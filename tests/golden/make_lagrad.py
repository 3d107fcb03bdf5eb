"""Record the reference's documented core-collapse run as a small fixture.

docs/sphinx/source/example_output/plummer.lagrad.dat is the lagrad.dat the
reference's documentation shows for examples/PlummerSphere.ini (N = 10^4
equal-mass Plummer sphere, THETASEMAX = 1, CMC_GAMMA = 0.1, AVEKERNEL = 20,
stopping at core collapse, STOPATCORECOLLAPSE = 1: N_core <= 100,
cmc_utils.c:527-532).  This keeps its final time (core collapse), its
number of steps, and the 1%, 10%, 50% and 90% Lagrange radii at a few
times, for tests/test_gpu_physics.py.

    python tests/golden/make_lagrad.py        # where the reference tree is mounted
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

SOURCE = os.path.join("docs", "sphinx", "source", "example_output", "plummer.lagrad.dat")
FRACTIONS = (0.01, 0.1, 0.5, 0.9)
TIMES = (0.0, 0.25, 0.5, 0.75, 1.0, 1.25, 1.5)
OUT = os.path.join(HERE, "plummer_lagrad.json")


def record(root: str) -> dict:
    path = os.path.join(root, SOURCE)
    lines = open(path).read().splitlines()
    header = [ln for ln in lines if ln.startswith("#")]
    cols = header[1].lstrip("#").split()  # "1:t 2:r(0.0001) ..."
    frac_col = {}
    for i, c in enumerate(cols):
        if c.startswith(f"{i + 1}:r("):
            frac_col[float(c[len(f"{i + 1}:r("):-1])] = i
    data = np.array([[float(x) for x in ln.split()] for ln in lines if ln and not ln.startswith("#")])
    t = data[:, 0]
    samples = []
    for tt in TIMES:
        row = data[int(np.argmin(np.abs(t - tt)))]
        samples.append({"t": float(row[0]), **{str(f): float(row[frac_col[f]]) for f in FRACTIONS}})
    return {"source": SOURCE, "steps": int(len(data)), "t_core_collapse": float(t[-1]),
            "fractions": list(FRACTIONS), "samples": samples}


if __name__ == "__main__":
    root = oracle.reference_root()
    if root is None:
        sys.exit("reference tree not present")
    rec = record(root)
    with open(OUT, "w") as fp:
        json.dump(rec, fp, indent=1)
        fp.write("\n")
    print(f"wrote {OUT}: {rec['steps']} steps, core collapse at t = {rec['t_core_collapse']}")
