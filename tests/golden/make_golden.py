"""Regenerate the golden fixtures in this directory.

taus113.json  -- draws of the reference's own taus113 generator: its
                 src/libs/taus113-v2.c is compiled in place (oracle/_ref, by
                 oracle.build_ref) and called through ctypes; plus the
                 known-answer value of its testjumping() (taus113-v2.c:272-292).
philox.json   -- Random123 philox4x32-10 known-answer vectors (Salmon et al.,
                 SC'11), the counter generator of the GPU kernels.

Run from the repository root where the reference tree is mounted:
    python tests/golden/make_golden.py
"""
import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


class TausState(C.Structure):
    _fields_ = [("z", C.c_ulong * 4)]


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference tree not found; cannot regenerate taus113.json")
    L = C.CDLL(oracle.REF_TAUS)
    L.reset_rng_t113_new.argtypes = [C.c_ulong, C.POINTER(TausState)]
    L.rng_t113_int_new.argtypes = [C.POINTER(TausState)]
    L.rng_t113_int_new.restype = C.c_ulong
    L.rng_t113_next_state.argtypes = [TausState]
    L.rng_t113_next_state.restype = TausState
    streams = {}
    for seed in (0, 1, 123456, 987654321, 4294967295):
        st = TausState()
        L.reset_rng_t113_new(seed, C.byref(st))
        streams[str(seed)] = [int(L.rng_t113_int_new(C.byref(st))) for _ in range(16)]
    st = TausState()
    L.reset_rng_t113_new(123456, C.byref(st))
    for _ in range(1 << 20):
        st = L.rng_t113_next_state(st)
    kat = int(L.rng_t113_int_new(C.byref(st)))
    json.dump({"source": "src/libs/taus113-v2.c compiled in place", "after_2_20": kat, "streams": streams},
              open(os.path.join(HERE, "taus113.json"), "w"), indent=1)
    cases = [
        {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
        {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF] * 2, "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
        {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], "key": [0xA4093822, 0x299F31D0],
         "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
    ]
    json.dump({"source": "Random123 philox4x32-10 known-answer vectors", "cases": cases},
              open(os.path.join(HERE, "philox.json"), "w"), indent=1)
    print("wrote taus113.json (KAT %d) and philox.json" % kat)


if __name__ == "__main__":
    main()
