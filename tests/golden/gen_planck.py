"""Generate planck_nbb.json: black-body group integrals from the reference's
own NormalizedBlackBody.cc (built into oracle/_ref/libnbb.so by
oracle/ref_build.py on a machine with the UMT source tree).

    python tests/golden/gen_planck.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    from oracle import ref_build
    from umt_gb300.problems import group_bounds, SPEED_LIGHT, RAD_CONSTANT
    out = ref_build.build()
    lib = C.CDLL(os.path.join(out, "libnbb.so"))
    lib.NBB_integrateBlackBodyGroups.restype = None
    cases = []
    for T in (0.05, 0.5, 1.0e-3, 3.0):
        for ngr in (1, 2, 16, 32):
            gnu = group_bounds(ngr)
            B = np.zeros(ngr)
            lib.NBB_integrateBlackBodyGroups(C.c_double(T), C.c_double(1.0),
                                             C.c_double(SPEED_LIGHT * RAD_CONSTANT), C.c_int(ngr),
                                             gnu.ctypes.data_as(C.c_void_p), B.ctypes.data_as(C.c_void_p))
            cases.append(dict(T=T, ngr=ngr, k=1.0, bnorm=SPEED_LIGHT * RAD_CONSTANT,
                              gnu=gnu.tolist(), B=B.tolist()))
    with open(os.path.join(HERE, "planck_nbb.json"), "w") as f:
        json.dump(dict(source="src/teton/misc/NormalizedBlackBody.cc NBB_integrateBlackBodyGroups",
                       cases=cases), f, indent=1)


if __name__ == "__main__":
    main()
