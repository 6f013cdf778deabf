"""CPU baseline of the integrator timings (measurement infrastructure, not
part of the product): the reference's own integrators, unmodified, with its
own C backend (tupan/lib/cffi_backend.py, built by cffi at import), on the
workload of `python -m tupan_gb300.runs integrators`: a Plummer sphere of n
equal masses without softening, base step eta, one untimed step, then
`steps` timed steps; ms per step on one core.

    python oracle/time_reference_integrators.py --ref baseline/_ref [--n 256]

Needs an installed reference tree and cffi with a C compiler (this runs on
the build machine; the GPU timings come from tupan_gb300.runs).
"""
import argparse
import json
import os
import sys
import tempfile
import time


HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TUPAN_REF"), help="installed reference tree")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--eta", type=float, default=1.0 / 64)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--methods", default="sia21h.dkd,sia21h.kdk,sia44h.kdk,sia21s.kdk,"
                                          "ahermite4,hermite6,sakura,nreg")
    a = ap.parse_args()
    if not a.ref:
        sys.exit("give --ref <reference tree> or set TUPAN_REF")
    os.environ.setdefault("HOME", tempfile.mkdtemp(prefix="tupan_home_"))
    sys.path.insert(0, os.path.abspath(a.ref))
    sys.path.insert(1, ROOT)
    from tupan_gb300.ics import plummer_arrays          # host-only, no GPU library
    from tupan.integrator import Integrator
    from tupan.lib import extensions
    from tupan.particles.allparticles import ParticleSystem
    d = plummer_arrays(a.n, 0.0, seed=a.seed)
    out = {"config": {"n": a.n, "eta": a.eta, "steps": a.steps, "eps2": 0.0, "seed": a.seed,
                      "backend": type(extensions.acc.kernel).__module__, "cores": 1},
           "ms_per_step": {}}
    for method in a.methods.split(","):
        ps = ParticleSystem(a.n)
        for k in ("mass", "rx", "ry", "rz", "vx", "vy", "vz"):
            getattr(ps, k)[...] = d[k]
        ps.eps2[...] = 0.0
        integ = Integrator(a.eta, 0.0, ps, method=method)
        integ.evolve_step(a.eta)
        t0 = time.perf_counter()
        for k in range(a.steps):
            integ.evolve_step((k + 2) * a.eta)
        out["ms_per_step"][method] = (time.perf_counter() - t0) / a.steps * 1e3
    print(json.dumps(out))


if __name__ == "__main__":
    main()
