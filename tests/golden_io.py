"""Loader for the golden fixtures written by tests/golden/make_golden.py."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz",
          "ax", "ay", "az", "jx", "jy", "jz")
CASES = ("sweep", "plummer", "binary", "edge")
PREFIXES = (1, 2, 3, 31, 33, 64, 65, 96)


def load(case):
    z = np.load(os.path.join(GOLDEN, "golden_%s.npz" % case))
    ps = {f: z["in_" + f] for f in FIELDS}
    calls = []
    for key in z["calls"]:
        key = str(key)
        name = key.split("_", 1)[1]
        sc = tuple(z["scalars_" + key])
        calls.append((key, name, sc))
    return z, ps, calls


def typed_scalars(name, sc):
    """Restore the integer scalars stored as float64 in the fixtures."""
    if name == "pnacc":
        return (int(sc[0]),) + tuple(float(x) for x in sc[1:])
    if name == "sakura":
        return (float(sc[0]), int(sc[1]))
    return tuple(float(x) for x in sc)
