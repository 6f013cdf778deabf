"""Loader for tests/golden/golden_integrators.npz (reference integrator runs)."""
import os

import numpy as np

from golden_io import GOLDEN

RUNS = ("ahermite2", "ahermite4", "hermite6", "hermite8", "sia21s.kdk", "sia21s.dkd",
        "sia21a.kdk", "sakura", "asakura", "nreg", "anreg",
        "sia22s.dkd", "sia43s.kdk", "sia44a.dkd", "sia45s.kdk", "sia46a.kdk", "sia67s.dkd", "sia69s.kdk",
        "sia21h.dkd", "sia21h.kdk", "sia22h.dkd", "sia44h.kdk", "sia69h.kdk")
# runs whose two-body subsystems go through the Kepler solver (transcendentals)
KEPLER_RUNS = ("sakura", "asakura", "sia21h.dkd", "sia21h.kdk", "sia22h.dkd", "sia44h.kdk", "sia69h.kdk")
RV = ("rx", "ry", "rz", "vx", "vy", "vz")


def load():
    return np.load(os.path.join(GOLDEN, "golden_integrators.npz"))


def run_config(z, method):
    eta, t_end, eps2, steps, t_final = z["cfg_" + method.replace(".", "_")]
    return float(eta), float(t_end), float(eps2), int(steps), float(t_final)


def initial_state(z, eps2):
    d = {k[3:]: z[k] for k in z.files if k.startswith("ic_")}
    d["eps2"] = np.full(len(d["mass"]), eps2)
    return d


def final_state(z, method):
    key = method.replace(".", "_")
    return np.stack([z["end_%s_%s" % (key, f)] for f in RV])


def final_ids(z, method):
    """Particle ids in the reference's final order (the h. split reorders)."""
    key = "end_%s_id" % method.replace(".", "_")
    return z[key] if key in z.files else None
