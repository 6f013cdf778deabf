"""Generate the golden fixtures in tests/golden/ from the reference C backend.

Run where a reference tree is available, its root in TUPAN_REF:

    make -f oracle/ref.mk REF=$TUPAN_REF
    TUPAN_REF=<reference root> python tests/golden/make_golden.py

The reference's own kernels (tupan/lib/src/*_kernel.c, compiled unmodified by
oracle/ref.mk into oracle/_ref/libtupan_ref_f64.so) are called through
oracle.oracle.ReferenceLib on seeded inputs; inputs and outputs are stored as
compressed .npz files.  The GPU machine has no reference tree, so these fixtures
carry the pin there.

Cases (the reference test suite, tupan/tests/test_extensions.py:28-127, asserts
nothing and uses unseeded inputs; these restate its shapes, seeded):
  sweep    n=96 particles, masses U(0,1), eps2=0, positions and velocities
           U(0,10) (test_extensions.py:28-36); outputs for i=all vs j=prefix
           and i=prefix vs j=all at prefix lengths 1,2,3,31,33,64,65,96
           (test_extensions.py:45-85); eta=1/64, PN order 7 with c=128,
           Sakura dt=1/64 with flags -2,-1,0,1,2.
  plummer  n=384 Plummer sphere, equal masses, per-particle eps2 = 0.5e-4.
  binary   n=64: 32 wide particles plus 16 pairs at separation ~1e-3 with
           eps2=0 (Sakura's Kepler branch, PN order 5/7 with c=1e2).
  edge     n=5 with two coincident particles (r2 = 0 for a distinct pair)
           and a massless particle.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import ReferenceLib, SPECS  # noqa: E402

FIELDS = SPECS["snap_crackle"][0]
PREFIXES = (1, 2, 3, 31, 33, 64, 65, 96)


def sweep_set(rng, n=96):
    ps = {f: rng.random(n) * 10 for f in FIELDS}
    ps["mass"] = rng.random(n)
    ps["eps2"] = np.zeros(n)
    return ps


def plummer_set(rng, n=384):
    x1 = rng.random(n)
    r = 1 / np.sqrt(x1 ** (-2.0 / 3.0) - 1)
    ct = 2 * rng.random(n) - 1
    st = np.sqrt(1 - ct * ct)
    ph = 2 * np.pi * rng.random(n)
    pos = np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct], 1) * (3 * np.pi / 16)
    vel = rng.normal(size=(n, 3)) * 0.5
    ps = {"mass": np.full(n, 1.0 / n), "eps2": np.full(n, 0.5e-4)}
    for k, c in enumerate("xyz"):
        ps["r" + c] = pos[:, k].copy()
        ps["v" + c] = vel[:, k].copy()
    for f in ("ax", "ay", "az", "jx", "jy", "jz"):
        ps[f] = rng.normal(size=n)
    return ps


def binary_set(rng, n=64):
    h = n // 2
    base = rng.normal(size=(h, 3))
    pos = np.concatenate([base, base + rng.normal(size=(h, 3)) * 1e-3])
    vel = np.concatenate([rng.normal(size=(h, 3)) * 0.3, rng.normal(size=(h, 3)) * 3])
    ps = {"mass": rng.random(n) / n, "eps2": np.zeros(n)}
    for k, c in enumerate("xyz"):
        ps["r" + c] = pos[:, k].copy()
        ps["v" + c] = vel[:, k].copy()
    for f in ("ax", "ay", "az", "jx", "jy", "jz"):
        ps[f] = rng.normal(size=n)
    return ps


def edge_set():
    ps = {f: np.zeros(5) for f in FIELDS}
    ps["mass"][:] = [0.5, 0.25, 0.25, 0.0, 1.0]
    ps["rx"][:] = [0.0, 1.0, 1.0, -2.0, 0.5]
    ps["ry"][:] = [0.0, 0.0, 0.0, 1.0, 3.0]
    ps["rz"][:] = [0.0, 0.0, 0.0, 0.0, -1.0]
    ps["vx"][:] = [0.0, 0.5, -0.5, 0.1, 0.0]
    ps["vy"][:] = [0.1, 0.0, 0.0, 0.0, 0.2]
    ps["vz"][:] = [0.0, 0.0, 0.3, 0.0, 0.0]
    ps["eps2"][:] = [1e-3, 0.0, 0.0, 1e-3, 0.0]
    for f in ("ax", "ay", "az", "jx", "jy", "jz"):
        ps[f][:] = np.linspace(-1, 1, 5)
    return ps


def pn_scalars(order, c):
    return (order,) + tuple((1.0 / c) ** k for k in range(1, 8))


def calls_for(case):
    """(kernel, scalars) pairs exercised on each case."""
    out = [("phi", ()), ("acc", ()), ("acc_jerk", ()), ("snap_crackle", ()),
           ("tstep", (1.0 / 64,))]
    if case == "sweep":
        out += [("pnacc", pn_scalars(7, 128.0))]
        out += [("sakura", (1.0 / 64, f)) for f in (-2, -1, 0, 1, 2)]
    elif case == "binary":
        out += [("pnacc", pn_scalars(5, 1e2)), ("pnacc", pn_scalars(7, 1e2))]
        out += [("sakura", (1.0 / 64, f)) for f in (-2, -1, 1, 2)]
        out += [("sakura", (0.3, 1))]
    elif case == "plummer":
        out += [("pnacc", pn_scalars(4, 1e2))]
        out += [("tstep", (0.01,))]
    elif case == "edge":
        out += [("pnacc", pn_scalars(7, 10.0))]
    return out


def main():
    ref = ReferenceLib()
    rng = np.random.default_rng(20261203)
    sets = {"sweep": sweep_set(rng), "plummer": plummer_set(rng),
            "binary": binary_set(rng), "edge": edge_set()}
    for case, ps in sets.items():
        store = {"in_" + f: ps[f] for f in FIELDS}
        calls = calls_for(case)
        names = []
        for k, (name, sc) in enumerate(calls):
            key = "%02d_%s" % (k, name)
            names.append(key)
            store["scalars_" + key] = np.array(sc, dtype=np.float64)
            res = ref.calc(name, ps, ps, *sc)
            store["out_" + key] = np.stack(res)
            if case == "sweep" and name != "sakura":
                for p in PREFIXES:
                    sub = {f: ps[f][:p] for f in FIELDS}
                    store["outJ%d_" % p + key] = np.stack(ref.calc(name, ps, sub, *sc))
                    store["outI%d_" % p + key] = np.stack(ref.calc(name, sub, ps, *sc))
        store["calls"] = np.array(names)
        path = os.path.join(HERE, "golden_%s.npz" % case)
        np.savez_compressed(path, **store)
        print("wrote", path, os.path.getsize(path), "bytes,", len(calls), "calls")


if __name__ == "__main__" and "--integrators" not in sys.argv and "--nreg-kepler" not in sys.argv:
    main()


# ---------------------------------------------------------------------------
# Integrator trajectories from the reference integrators themselves.
# ---------------------------------------------------------------------------
INTEGRATOR_RUNS = (
    # method, eta, t_end, eps2
    ("ahermite2", 0.01, 1.0 / 64, 1e-3),
    ("ahermite4", 0.01, 1.0 / 32, 1e-3),
    ("hermite6", 1.0 / 128, 1.0 / 32, 1e-3),
    ("hermite8", 1.0 / 128, 1.0 / 64, 1e-3),
    ("sia21s.kdk", 1.0 / 256, 1.0 / 32, 1e-3),
    ("sia21s.dkd", 1.0 / 256, 1.0 / 32, 1e-3),
    ("sia21a.kdk", 0.01, 1.0 / 32, 1e-3),
    ("sakura", 1.0 / 128, 1.0 / 64, 0.0),
    ("asakura", 0.01, 1.0 / 64, 0.0),
    ("nreg", 1.0 / 256, 1.0 / 32, 1e-3),
    ("anreg", 1.0 / 256, 1.0 / 32, 1e-3),
    ("sia22s.dkd", 1.0 / 256, 1.0 / 32, 1e-3),
    ("sia43s.kdk", 1.0 / 256, 1.0 / 32, 1e-3),
    ("sia44a.dkd", 0.01, 1.0 / 32, 1e-3),
    ("sia45s.kdk", 1.0 / 256, 1.0 / 64, 1e-3),
    ("sia46a.kdk", 0.01, 1.0 / 64, 1e-3),
    ("sia67s.dkd", 1.0 / 128, 1.0 / 64, 1e-3),
    ("sia69s.kdk", 1.0 / 128, 1.0 / 64, 1e-3),
    # hierarchical split; eps2 = 0 so that two-body subsystems take the
    # Kepler solver's unsoftened branch, whose retries always terminate
    ("sia21h.dkd", 1.0 / 128, 1.0 / 32, 0.0),
    ("sia21h.kdk", 1.0 / 128, 1.0 / 32, 0.0),
    ("sia22h.dkd", 1.0 / 128, 1.0 / 32, 1e-3),
    ("sia44h.kdk", 1.0 / 128, 1.0 / 64, 0.0),
    ("sia69h.kdk", 1.0 / 128, 1.0 / 64, 0.0),
)


def integrator_ics(n=48, seed=7):
    rng = np.random.default_rng(seed)
    d = {"mass": rng.random(n) / n}
    for c in "xyz":
        d["r" + c] = rng.normal(size=n)
        d["v" + c] = rng.normal(size=n) * 0.3
    return d


def reference_trajectories(ref_root=None):
    """Run the reference integrators (imported from the reference tree, with
    HOME redirected for its cffi build cache) on the same initial state."""
    import tempfile
    ref_root = ref_root or os.environ["TUPAN_REF"]
    os.environ["HOME"] = tempfile.mkdtemp(prefix="tupan_home_")
    sys.path.insert(0, ref_root)
    from tupan.integrator import Integrator
    from tupan.particles.allparticles import ParticleSystem
    ics = integrator_ics()
    n = len(ics["mass"])
    store = {"ic_" + k: v for k, v in ics.items()}
    for method, eta, t_end, eps2 in INTEGRATOR_RUNS:
        ps = ParticleSystem(n)
        for k, v in ics.items():
            getattr(ps, k)[...] = v
        ps.eps2[...] = eps2
        integ = Integrator(eta, 0.0, ps, method=method)
        steps = 0
        while abs(integ.time) < abs(t_end):
            integ.evolve_step(t_end)
            steps += 1
        out = integ.particle_system
        key = method.replace(".", "_")
        store["cfg_" + key] = np.array([eta, t_end, eps2, steps, integ.time])
        for f in ("rx", "ry", "rz", "vx", "vy", "vz"):
            store["end_%s_%s" % (key, f)] = np.array(getattr(out, f))
        store["end_%s_id" % key] = np.array(out.id, dtype=np.int64)
        print(method, steps, "steps to", integ.time)
    path = os.path.join(HERE, "golden_integrators.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__" and "--integrators" in sys.argv:
    reference_trajectories()


# ---------------------------------------------------------------------------
# NREG_X / NREG_V and the Kepler pair solver (libtupan.h:152-201, 231-246).
#
#   python tests/golden/make_golden.py --nreg-kepler
#
# golden_nreg.npz: nreg_x and nreg_v of the reference on the inputs of the
# four kernel cases above (read back from their fixtures) at dt = 0, 1/64 and
# -0.3, plus the i=all vs j=prefix / i=prefix vs j=all sweeps on "sweep" at
# dt = 1/64.
# golden_kepler.npz: kepler_solver_kernel of the reference, one call per
# pair, on seeded pairs: bound orbits (e up to 0.95, apocentre start),
# hyperbolic encounters, pairs with eps2 = (1e-6 a)^2 / 2, a pair at r = 0
# and a massless companion; dt = 1/64, 0.37 and -0.5.  Softened pairs that
# need more sub-steps than the GPU solver's bounds are not in the fixture
# (the reference's retry loops are unbounded; see tests/test_gpu_nreg_kepler.py).
# ---------------------------------------------------------------------------
NREG_DTS = (0.0, 1.0 / 64, -0.3)
KEPLER_DTS = (1.0 / 64, 0.37, -0.5)


def kepler_pairs(rng, npairs, kind, soft=0.0):
    p8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")
    ps = {f: np.zeros(2 * npairs) for f in p8}
    for p in range(npairs):
        m1, m2 = rng.random() * 0.5 + 0.01, rng.random() * 0.5 + 0.01
        a = np.exp(rng.uniform(np.log(1e-3), np.log(1.0)))
        e = 0.95 * np.sqrt(rng.random())
        M = m1 + m2
        if kind == "hyper":
            r = a
            v = np.sqrt(2 * M / r) * (1.2 + rng.random())
        else:
            r = a * (1 + e)
            v = np.sqrt(M * (1 - e) / (a * (1 + e)))
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        rr, vv = q @ np.array([r, 0.0, 0.0]), q @ np.array([0.0, v, 0.0])
        cm, cv = rng.normal(size=3), rng.normal(size=3) * 0.3
        ri, rj = cm + m2 / M * rr, cm - m1 / M * rr
        vi, vj = cv + m2 / M * vv, cv - m1 / M * vv
        for k, c in enumerate("xyz"):
            ps["r" + c][2 * p], ps["r" + c][2 * p + 1] = ri[k], rj[k]
            ps["v" + c][2 * p], ps["v" + c][2 * p + 1] = vi[k], vj[k]
        ps["mass"][2 * p], ps["mass"][2 * p + 1] = m1, m2
        ps["eps2"][2 * p] = ps["eps2"][2 * p + 1] = (a * soft) ** 2 / 2
    return ps


def kepler_edge_pairs():
    # a pair at r = 0 (centre of mass drifts only) and a massless companion
    p8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")
    ps = {f: np.zeros(4) for f in p8}
    ps["mass"][:] = [0.3, 0.2, 0.5, 0.0]
    ps["rx"][:] = [1.0, 1.0, -0.5, -0.4]
    ps["ry"][:] = [0.5, 0.5, 0.2, 0.2]
    ps["vx"][:] = [0.1, -0.2, 0.0, 0.0]
    ps["vy"][:] = [0.0, 0.3, 0.0, 1.5]
    return ps


def nreg_kepler():
    ref = ReferenceLib()
    store = {}
    for case in ("sweep", "plummer", "binary", "edge"):
        z = np.load(os.path.join(HERE, "golden_%s.npz" % case))
        ps = {f: z["in_" + f] for f in FIELDS}
        for dt in NREG_DTS:
            for name in ("nreg_x", "nreg_v"):
                key = "%s_%s_%r" % (case, name, dt)
                store[key] = np.stack(ref.calc(name, ps, ps, dt))
                if case == "sweep" and dt == 1.0 / 64:
                    for p in PREFIXES:
                        sub = {f: ps[f][:p] for f in FIELDS}
                        store["J%d_" % p + key] = np.stack(ref.calc(name, ps, sub, dt))
                        store["I%d_" % p + key] = np.stack(ref.calc(name, sub, ps, dt))
    path = os.path.join(HERE, "golden_nreg.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, os.path.getsize(path), "bytes")

    rng = np.random.default_rng(5)
    sets = {"bound": kepler_pairs(rng, 16, "bound"), "hyper": kepler_pairs(rng, 16, "hyper"),
            "soft": kepler_pairs(rng, 16, "bound", soft=1e-6), "edge": kepler_edge_pairs()}
    store = {}
    for kind, ps in sets.items():
        for f, v in ps.items():
            store["in_%s_%s" % (kind, f)] = v
        for dt in KEPLER_DTS:
            store["out_%s_%r" % (kind, dt)] = np.stack(ref.kepler(ps, dt))
    path = os.path.join(HERE, "golden_kepler.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__" and "--nreg-kepler" in sys.argv:
    nreg_kepler()
