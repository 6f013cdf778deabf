"""Golden final state of the adaptive-Hermite configuration (run here once).

Plummer N = 4096 (tupan_gb300.ics.plummer_arrays, seed 4096, eps = 0.01 so
per-particle eps2 = 5e-5 and pair e2 = 1e-4), ahermite4 with eta = 0.01 from
t = 0 to t = 1/8, integrated by the CPU restatement of the reference
integrator (oracle/integrators.py, bit-identical to tupan/integrator/
hermite.py with the reference C kernels).  About 4100 block steps; ~11 min
on 8 cores.

    python tests/golden/make_config1.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import integrators as oi  # noqa: E402
from tupan_gb300.ics import plummer_arrays  # noqa: E402

N, EPS, SEED, ETA, T_END = 4096, 0.01, 4096, 0.01, 0.125


def main():
    # The initial state is stored too: numpy's sin/cos/power differ in the last
    # bits between CPU architectures, and 4500 chaotic steps amplify that.
    d = plummer_arrays(N, EPS, seed=SEED)
    integ = oi.integrator("ahermite4", ETA, oi.make_ps(d), oi.Kernels(nthreads=os.cpu_count() or 4))
    t0 = time.time()
    steps = 0
    while abs(integ.t_curr) < abs(T_END):
        integ.evolve_step(T_END)
        steps += 1
    out = {f: integ.ps[f] for f in ("rx", "ry", "rz", "vx", "vy", "vz")}
    out.update({"ic_" + k: v for k, v in d.items()})
    np.savez_compressed(os.path.join(HERE, "golden_config1.npz"), steps=steps, t_final=integ.t_curr,
                        n=N, eps=EPS, seed=SEED, eta=ETA, t_end=T_END, **out)
    print("steps", steps, "seconds", time.time() - t0)


if __name__ == "__main__":
    main()
