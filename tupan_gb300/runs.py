"""Named workload runs: the precision, differentiation and binary-cluster
configurations, each reporting a JSON summary.

    python -m tupan_gb300.runs precision      # Plummer-Salpeter N=65536 SIA21
    python -m tupan_gb300.runs adjoint        # N=16384 leapfrog gradients
    python -m tupan_gb300.runs binaries       # 2048 + 64 binaries, PN + Sakura
    python -m tupan_gb300.runs ensemble       # 512 clusters, Hermite-6, CUDA graph
    python -m tupan_gb300.runs kernels --n N  # per-kernel device time, ds32 and FP64
    python -m tupan_gb300.runs integrators    # ms per step of the integrators, N=256
    python -m tupan_gb300.runs snapshots      # snapshot/worldline file cost, N=65536 SIA21

All inputs are seeded synthetic Plummer spheres (tupan_gb300.ics).
"""
import argparse
import json
import math
import time

import numpy as np
import torch

from . import _native, autodiff
from .ics import Salpeter, make_binary, plummer_arrays
from .integrator import Integrator
from .lib import extensions
from .particles import ParticleSystem

RV = ("rx", "ry", "rz", "vx", "vy", "vz")


def energy(ps):
    """Total energy K + U with the FP64 Phi kernel (body.py:259-306)."""
    extensions.Phi("CUDA", "float64").calc(ps, ps)
    k = 0.5 * float((ps.mass * (ps.vx ** 2 + ps.vy ** 2 + ps.vz ** 2)).sum())
    u = 0.5 * float((ps.mass * ps.phi).sum())
    return k + u


def force_error(ps):
    """Per-particle |a_ds32 - a_fp64| / |a_fp64| on the current positions."""
    a64 = np.stack([o.cpu().numpy() for o in extensions.Acc("CUDA", "float64").calc(ps, ps)])
    a32 = np.stack([o.cpu().numpy() for o in extensions.Acc("CUDA", "ds32").calc(ps, ps)])
    r = np.sqrt(((a32 - a64) ** 2).sum(0)) / np.sqrt((a64 ** 2).sum(0))
    return {"max": float(r.max()), "p999": float(np.percentile(r, 99.9)),
            "p99": float(np.percentile(r, 99)), "median": float(np.median(r))}


def precision_run(n=65536, steps=128, dt=1.0 / 1024, seed=20261203, probe_every=32):
    """Shared-step SIA21 kdk leapfrog, split FP32 against FP64."""
    d = plummer_arrays(n, 1e-3, imf=Salpeter(0.1, 100.0), seed=seed)
    out = {"config": {"n": n, "imf": "salpeter [0.1,100]", "eps2_pair": 1e-6, "method": "sia21s.kdk",
                      "dt": dt, "steps": steps, "tstep_eta": dt}}
    for prec in ("ds32", "float64"):
        extensions.set_precision(prec)
        ps = ParticleSystem.from_arrays(**d)
        e0 = energy(ps)
        integ = Integrator(dt, 0.0, ps, method="sia21s.kdk")
        probes = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(steps):
            integ.evolve_step((s + 1) * dt)
            integ.particle_system.set_tstep(integ.particle_system, dt)
            if prec == "ds32" and probe_every and (s + 1) % probe_every == 0:
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                probes.append({"step": s + 1, "force_error": force_error(integ.particle_system)})
                t0 += time.perf_counter() - t1
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        ps = integ.particle_system
        e1 = energy(ps)
        out[prec] = {"e0": e0, "e1": e1, "rel_energy_error": abs((e1 - e0) / e0),
                     "ms_per_step": 1e3 * wall / steps,
                     "min_tstep_last": float(ps.tstep.abs().min()),
                     "final": {f: getattr(ps, f).cpu().numpy() for f in RV}}
        if probes:
            out[prec]["force_error_probes"] = probes
    extensions.set_precision("float64")
    ps0 = ParticleSystem.from_arrays(**d)
    out["force_error_step0"] = force_error(ps0)
    fa, fb = out["ds32"].pop("final"), out["float64"].pop("final")
    dpos = np.sqrt(sum((fa[f] - fb[f]) ** 2 for f in ("rx", "ry", "rz")))
    out["trajectory_difference"] = {"max_abs_position": float(dpos.max()), "median": float(np.median(dpos))}
    out["energy_drift_ratio_ds32_over_fp64"] = out["ds32"]["rel_energy_error"] / max(out["float64"]["rel_energy_error"], 1e-300)
    return out


def adjoint_run(n=16384, steps=64, dt=1.0 / 256, seed=16384, checkpoint_every=8, ncoords=32):
    """Gradients of a trajectory loss by the Acc adjoint, checked by FP64
    central finite differences.  Three arithmetics for the forward and the
    adjoint: ds32 (the split-FP32 forces, <= 1e-6 per particle, with the
    double-single adjoint), ds32x (double-single forces and adjoint, ~1e-12)
    and float64."""
    d = plummer_arrays(n, 0.01, seed=seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    r0 = torch.tensor(np.stack([d["rx"], d["ry"], d["rz"]]), dtype=torch.float64, device=dev)
    v0 = torch.tensor(np.stack([d["vx"], d["vy"], d["vz"]]), dtype=torch.float64, device=dev)
    m0 = torch.tensor(d["mass"], dtype=torch.float64, device=dev)
    e2 = torch.tensor(d["eps2"], dtype=torch.float64, device=dev)
    rng = np.random.default_rng(seed)
    noise = torch.tensor(rng.lognormal(0.0, 0.01, n), dtype=torch.float64, device=dev)
    with torch.no_grad():
        target, _ = autodiff.leapfrog(r0, v0, m0 * noise, e2, dt, steps, "float64", 0)

    def loss(r, v, m, prec, ck):
        rf, _ = autodiff.leapfrog(r, v, m, e2, dt, steps, prec, ck)
        return autodiff.loss_to_target(rf, target)

    out = {"config": {"n": n, "steps": steps, "dt": dt, "eps2_pair": 1e-4, "checkpoint_every": checkpoint_every,
                      "target": "same ICs, masses x lognormal(sigma=0.01), not renormalised, FP64 run"}}
    grads = {}
    for prec in ("ds32", "ds32x", "float64"):
        # untimed one-step pass: first use of the torch and library kernels
        # (loading them on a fresh machine takes seconds)
        rw = r0.clone().requires_grad_(True)
        rfw, _ = autodiff.leapfrog(rw, v0, m0, e2, dt, 1, prec, checkpoint_every)
        autodiff.loss_to_target(rfw, target).backward()
        torch.cuda.synchronize()
        r = r0.clone().requires_grad_(True)
        v = v0.clone().requires_grad_(True)
        m = m0.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L = loss(r, v, m, prec, checkpoint_every)
        L.backward()
        torch.cuda.synchronize()
        grads[prec] = (r.grad, v.grad, m.grad)
        out[prec] = {"loss": float(L.detach()), "seconds_forward_backward": time.perf_counter() - t0,
                     "peak_mem_mb": torch.cuda.max_memory_allocated() / 2 ** 20}
    for prec in ("ds32", "ds32x"):
        rel = [float((a - b).norm() / b.norm()) for a, b in zip(grads[prec], grads["float64"])]
        out[prec + "_vs_fp64_adjoint_rel_norm"] = {"r": rel[0], "v": rel[1], "m": rel[2]}
    worst64, worst32, worst32x, within, within32x, checks = 0.0, 0.0, 0.0, 0, 0, []
    with torch.no_grad():
        for q in range(ncoords):
            which = ("r", "v", "m")[q % 3]
            base = {"r": r0, "v": v0, "m": m0}[which]
            idx = tuple(int(rng.integers(0, s)) for s in base.shape)
            scale = max(abs(float(base[idx])), 0.1) if which != "m" else float(base[idx])

            def central(step):
                args_p = {"r": r0, "v": v0, "m": m0}
                args_m = dict(args_p)
                bp, bm = base.clone(), base.clone()
                bp[idx] += step
                bm[idx] -= step
                args_p[which], args_m[which] = bp, bm
                return float(loss(args_p["r"], args_p["v"], args_p["m"], "float64", 0)
                             - loss(args_m["r"], args_m["v"], args_m["m"], "float64", 0)) / (2 * step)

            # Step ladder h = scale x 10^-k: small steps are dominated by the
            # rounding noise of the FP64 trajectories, large ones by the h^2
            # truncation of close encounters.  Richardson with ratio 10,
            # R(h) = (100 D(h) - D(10 h)) / 99, removes the h^2 term; the
            # estimate kept is the one that agrees best with its neighbour,
            # and that disagreement is the finite difference's own error.
            D = {k: central(scale * 10.0 ** -k) for k in FD_LADDER}
            R = {k: (100.0 * D[k] - D[k - 1]) / 99.0 for k in FD_LADDER[1:]}
            pairs = [(k, k + 1) for k in FD_LADDER[1:-1]]
            kb, kn = min(pairs, key=lambda p: abs(R[p[0]] - R[p[1]]))
            fd, spread = R[kb], abs(R[kb] - R[kn])
            k = "rvm".index(which)
            g64, g32, g32x = (float(grads[p][k][idx]) for p in ("float64", "ds32", "ds32x"))
            den = max(abs(fd), 1e-300)
            e64, e32, e32x = abs(g64 - fd) / den, abs(g32 - fd) / den, abs(g32x - fd) / den
            worst64, worst32, worst32x = max(worst64, e64), max(worst32, e32), max(worst32x, e32x)
            within += abs(g64 - fd) <= max(1e-6 * abs(fd), 2.0 * spread)
            within32x += abs(g32x - fd) <= max(1e-6 * abs(fd), 2.0 * spread)
            checks.append({"coord": which + str(idx), "fd": fd, "h": scale * 10.0 ** -kb,
                           "fd_spread_rel": spread / den, "adjoint_fp64": g64, "adjoint_ds32": g32,
                           "adjoint_ds32x": g32x, "rel_error_fp64": e64, "rel_error_ds32x": e32x})
    out["finite_difference"] = {
        "coordinates": ncoords,
        "method": "central differences at h = scale x 10^-k (k = %s), Richardson ratio 10, "
                  "most self-consistent step kept" % ",".join(map(str, FD_LADDER)),
        "max_rel_error_fp64_adjoint": worst64, "max_rel_error_ds32_adjoint": worst32,
        "max_rel_error_ds32x_adjoint": worst32x,
        "median_rel_error_fp64_adjoint": float(np.median([c["rel_error_fp64"] for c in checks])),
        "median_rel_error_ds32x_adjoint": float(np.median([c["rel_error_ds32x"] for c in checks])),
        "fp64_within_max(1e-6, 2 x fd spread)": "%d of %d" % (within, ncoords),
        "ds32x_within_max(1e-6, 2 x fd spread)": "%d of %d" % (within32x, ncoords),
        "samples": sorted(checks, key=lambda c: -c["rel_error_fp64"])[:6]}
    return out


# finite-difference step exponents of the adjoint check (h = scale x 10^-k)
FD_LADDER = (3, 4, 5, 6)


def binaries_run(nbg=2048, nbin=64, t_end=1.0 / 16, dt=1.0 / 1024, clight=1e4, pn_order=5, seed=2176,
                 compare_fp64=True):
    """Plummer background plus hard binaries: Sakura Kepler-drift steps (FP64)
    with a post-Newtonian kick (split FP32 PNAcc) split around them
    (kick tau/2, Sakura step tau, kick tau/2).  With compare_fp64 the same
    run with the FP64 PNAcc gives what the split-FP32 PN bound does to the
    binaries: the spread of their final separations and of all positions."""
    from .integrator.sakura import sakura_step
    d = plummer_arrays(nbg, 0.0, seed=seed)
    rng = np.random.default_rng(seed + 1)
    host = rng.choice(nbg, nbin, replace=False)
    cols = {k: list(d[k]) for k in ("mass", "rx", "ry", "rz", "vx", "vy", "vz")}
    mpart = 1.0 / (nbg + nbin)
    for k in range(nbg):
        cols["mass"][k] = mpart
    semis, eccs = [], []
    for h in host:
        a = math.exp(rng.uniform(math.log(1e-4), math.log(1e-3)))
        e = 0.9 * math.sqrt(rng.random())
        ms, rr, vv = make_binary(mpart, mpart, a, e, rng)
        semis.append(a)
        eccs.append(e)
        com_r = np.array([d["rx"][h], d["ry"][h], d["rz"][h]])
        com_v = np.array([d["vx"][h], d["vy"][h], d["vz"][h]])
        for c, ax in enumerate("xyz"):
            cols["r" + ax][h] = com_r[c] + rr[0][c]
            cols["v" + ax][h] = com_v[c] + vv[0][c]
            cols["r" + ax].append(com_r[c] + rr[1][c])
            cols["v" + ax].append(com_v[c] + vv[1][c])
        cols["mass"].append(mpart)
    n = nbg + nbin
    arrays = {k: np.array(v) for k, v in cols.items()}
    arrays["eps2"] = np.zeros(n)
    extensions.set_precision("float64")
    extensions.clight.pn_order = pn_order
    extensions.clight.clight = clight
    steps = int(round(t_end / dt))

    def run(prec):
        pn = extensions.PNAcc("CUDA", prec)
        ps = ParticleSystem.from_arrays(**arrays)

        def pn_kick(ps, tau):
            pn.calc(ps, ps)
            ps.vx += ps.pnax * tau
            ps.vy += ps.pnay * tau
            ps.vz += ps.pnaz * tau

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            pn_kick(ps, dt / 2)
            ps = sakura_step(ps, dt)
            pn_kick(ps, dt / 2)
        torch.cuda.synchronize()
        return ps, time.perf_counter() - t0

    def separations(ps):
        sep = []
        for k, h in enumerate(host):
            j = nbg + k
            dx = [float(getattr(ps, "r" + ax)[h] - getattr(ps, "r" + ax)[j]) for ax in "xyz"]
            sep.append(math.sqrt(sum(x * x for x in dx)))
        return np.array(sep)

    e0 = energy(ParticleSystem.from_arrays(**arrays))
    ps, wall = run("ds32")
    status = _native.sync_status(torch.cuda.current_stream().cuda_stream)
    e1 = energy(ps)
    sep = separations(ps)
    extra = {}
    if compare_fp64:
        ps64, wall64 = run("float64")
        status |= _native.sync_status(torch.cuda.current_stream().cuda_stream)
        sep64 = separations(ps64)
        dr = max(float((getattr(ps, "r" + ax) - getattr(ps64, "r" + ax)).abs().max()) for ax in "xyz")
        extra = {"fp64_pnacc": {"ms_per_step": 1e3 * wall64 / steps,
                                "rel_energy_error_newtonian": abs((energy(ps64) - e0) / e0)},
                 "ds32_vs_fp64": {"max_separation_difference_over_a":
                                      float(np.max(np.abs(sep - sep64) / np.array(semis))),
                                  "max_position_difference": dr}}
    return {"config": {"background": nbg, "binaries": nbin, "n": n, "a_range": [1e-4, 1e-3],
                       "e": "0.9*sqrt(u)", "eps2": 0.0, "pn_order": pn_order, "clight": clight,
                       "dt": dt, "t_end": t_end, "scheme": "PN kick dt/2, sakura_step dt, PN kick dt/2",
                       "pnacc_precision": "ds32", "sakura_precision": "float64"},
            "steps": steps, "ms_per_step": 1e3 * wall / steps, "kepler_status": status,
            "rel_energy_error_newtonian": abs((e1 - e0) / e0),
            "binary_separation_over_a": {"min": float(min(s / a for s, a in zip(sep, semis))),
                                         "max": float(max(s / a for s, a in zip(sep, semis)))},
            **extra}


def ensemble_run(nclusters=512, steps=16, dt=1.0 / 1024, base_seed=512, compare_fp64=True):
    """512 Plummer clusters (N log-uniform in [64, 8192]), 6th-order Hermite
    with a shared step, every force evaluation one segmented launch, one
    step captured in a CUDA graph and replayed.  With compare_fp64 the same
    steps are taken with the FP64 kernels (eagerly) and the per-cluster
    energy errors of the two are compared: the split-FP32 AccJerk and
    SnapCrackle bounds against what they do to the integrator."""
    from .ensemble import Ensemble, random_ensemble
    cl = random_ensemble(nclusters, base_seed=base_seed)
    ens = Ensemble(cl, prec="ds32")
    e0 = ens.energy()
    # per-kernel throughput (after the autotuning first calls)
    ens.acc_jerk()
    ens.snap_crackle()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    ens.acc_jerk()
    ev[1].record()
    ens.snap_crackle()
    ev[2].record()
    torch.cuda.synchronize()
    aj_ms, sc_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    # eager steps
    t0 = time.perf_counter()
    for _ in range(2):
        ens.hermite_step(dt)
    torch.cuda.synchronize()
    eager_ms = 1e3 * (time.perf_counter() - t0) / 2
    ens.capture(dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.replay(steps)
    torch.cuda.synchronize()
    graph_ms = 1e3 * (time.perf_counter() - t0) / steps
    e1 = ens.energy()
    de = np.abs((e1 - e0) / e0)
    total_steps = steps + 3
    out = {"config": {"clusters": nclusters, "n_range": [64, 8192], "total_particles": int(ens.ps.n),
                      "sum_n2": ens.interactions, "eps2_pair": 1e-4, "method": "hermite6 shared step",
                      "dt": dt, "steps": total_steps, "precision": "ds32"},
           "acc_jerk": {"ms": aj_ms, "gint_s": ens.interactions / (aj_ms * 1e-3) / 1e9},
           "snap_crackle": {"ms": sc_ms, "gint_s": ens.interactions / (sc_ms * 1e-3) / 1e9},
           "ms_per_step_eager": eager_ms, "ms_per_step_graph": graph_ms,
           "gint_s_per_step_graph": 3 * 2 * ens.interactions / (graph_ms * 1e-3) / 1e9,
           "energy_error": {"median": float(np.median(de)), "max": float(de.max())}}
    if compare_fp64:
        ref = Ensemble(cl, prec="float64")
        f0 = ref.energy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(total_steps):
            ref.hermite_step(dt)
        torch.cuda.synchronize()
        f1 = ref.energy()
        df = np.abs((f1 - f0) / f0)
        out["fp64"] = {"ms_per_step_eager": 1e3 * (time.perf_counter() - t0) / total_steps,
                       "energy_error": {"median": float(np.median(df)), "max": float(df.max())}}
        # per cluster: how far apart the two runs' final energies are
        diff = np.abs((e1 - f1) / f1)
        out["energy_ds32_vs_fp64_at_end"] = {"median": float(np.median(diff)), "max": float(diff.max())}
    return out


KERNEL_SCALARS = {"tstep": (1.0 / 1024,), "sakura": (1.0 / 1024, 1)}
# reference flop counts per interaction (<kernel>_kernel_common.h, last line of each core)
KERNEL_FLOP = {"phi": 14, "acc": 20, "acc_jerk": 42, "snap_crackle": 114, "tstep": 42}


def kernels_run(n=65536, reps=5, kernels="phi,acc,acc_jerk,snap_crackle,tstep,pnacc",
                precisions="ds32,float64", seed=20261203):
    """Per-kernel device time on a Plummer-Salpeter sphere (eps = 1e-3,
    Salpeter masses in [0.1, 100]): one untimed call, then `reps` calls each
    bracketed by CUDA events on the launching stream; median ms and Gint/s.
    Inputs of SnapCrackle (a, j) come from one FP64 AccJerk call.  PNAcc runs
    at order 5 with c = 1e4, Tstep with eta = 1/1024, Sakura with dt = 1/1024."""
    d = plummer_arrays(n, 1e-3, imf=Salpeter(0.1, 100.0), seed=seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    T = {k: torch.tensor(v, dtype=torch.float64, device=dev) for k, v in d.items()}
    for k in ("ax", "ay", "az", "jx", "jy", "jz"):
        T[k] = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    ptr = lambda names: [T[k].data_ptr() for k in names]  # noqa: E731
    _native.call_device("acc_jerk", n, ptr(_native.P8), n, ptr(_native.P8), (),
                        ptr(("ax", "ay", "az", "jx", "jy", "jz")), _native.PREC_FP64, stream)
    clight = extensions.Clight()
    clight.pn_order, clight.clight = 5, 1e4
    scal = dict(KERNEL_SCALARS)
    scal["pnacc"] = (clight.pn_order,) + tuple(getattr(clight, "inv%d" % k) for k in range(1, 8))
    out = {"config": {"n": n, "interactions": n * n, "reps": reps, "imf": "salpeter [0.1,100]",
                      "eps2_pair": 1e-6, "seed": seed}, "kernels": {}}
    for name in kernels.split(","):
        fields, _, outs = _native.SPECS[name]
        o = [torch.empty(n, dtype=torch.float64, device=dev) for _ in outs]
        for p in precisions.split(","):
            prec = autodiff.PREC[p]

            def call():
                _native.call_device(name, n, ptr(fields), n, ptr(fields), scal.get(name, ()),
                                    [x.data_ptr() for x in o], prec, stream)
            call()
            ms = []
            for _ in range(reps):
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                ev[0].record()
                call()
                ev[1].record()
                ev[1].synchronize()
                ms.append(ev[0].elapsed_time(ev[1]))
            med = float(np.median(ms))
            rec = {"ms": med, "gint_s": n * n / (med * 1e-3) / 1e9}
            if name in KERNEL_FLOP:
                rec["tflops_ref_counted"] = rec["gint_s"] * KERNEL_FLOP[name] / 1e3
            out["kernels"]["%s_%s" % (name, p)] = rec
    return out


def integrators_run(n=256, steps=8, methods="sia21h.dkd,sia21h.kdk,sia44h.kdk,sia21s.kdk,"
                    "ahermite4,hermite6,sakura,nreg", eta=1.0 / 64, seed=1):
    """Wall-clock ms per step (base step eta, one step per evolve_step call)
    of the GPU integrators in FP64 on a Plummer sphere of n equal-mass
    particles without softening (the reference's SIA/Sakura setting): one
    untimed step, then `steps` timed steps, synchronised on both sides.
    Hierarchical SIA methods are timed with the native recursion
    (tg_sia_h_step) and with the Python one; `levels` counts the time-step
    levels of one step (Tstep calls)."""
    from .integrator import sia
    extensions.set_precision("float64")
    d = plummer_arrays(n, 0.0, seed=seed)
    d["eps2"] = np.zeros(n)
    out = {"config": {"n": n, "eta": eta, "steps": steps, "eps2": 0.0, "seed": seed,
                      "ics": "plummer, equal masses, henon units", "precision": "float64"},
           "ms_per_step": {}}
    for method in methods.split(","):
        variants = [("", True)]
        if method[5:6] == "h":
            variants = [("", True), (" python", False)]
        for tag, native in variants:
            ps = ParticleSystem.from_arrays(**d)
            integ = Integrator(eta, 0.0, ps, method=method)
            if isinstance(integ.integrator, sia.SIA):
                integ.integrator.native_h = native
            integ.evolve_step(eta)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push(method + tag.replace(" ", "_"))   # ncu --nvtx-include <name>/
            t0 = time.perf_counter()
            for k in range(steps):
                integ.evolve_step((k + 2) * eta)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            out["ms_per_step"][method + tag] = (time.perf_counter() - t0) / steps * 1e3
    return out


def snapshots_run(n=65536, steps=16, dt=1.0 / 1024, seed=20261203):
    """Cost of the snapshot files (tupan_gb300.io) for the Plummer-Salpeter
    set of the precision configuration: one snapshot dump written
    synchronously and through the background writer (time until the call
    returns, and until the file is complete), the load back (checked
    bit-equal), and the wall-clock ms per step of sia21s.kdk in split FP32
    without a dumpper, with a per-step worldline dump written synchronously,
    and with it written by the background writer (dump_freq 1: every
    particle is dumped every step)."""
    import os
    import shutil
    import tempfile
    from .io import IO
    extensions.set_precision("ds32")
    d = plummer_arrays(n, 1e-3, imf=Salpeter(0.1, 100.0), seed=seed)
    tmp = tempfile.mkdtemp(prefix="tupan_snap_")
    out = {"config": {"n": n, "steps": steps, "dt": dt, "seed": seed, "method": "sia21s.kdk",
                      "precision": "ds32", "record_bytes": 96}}
    try:
        ps = ParticleSystem.from_arrays(**d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ps._real[:, :8].cpu()                       # the process's first device-to-host copy
        t1 = time.perf_counter()
        IO(os.path.join(tmp, "warm.hdf5"), "a").dump_snapshot(ps)
        t2 = time.perf_counter()
        out["first_d2h_ms"], out["first_dump_ms"] = (t1 - t0) * 1e3, (t2 - t1) * 1e3
        for tag, bg in (("sync", False), ("background", True)):
            path = os.path.join(tmp, tag + ".hdf5")
            io = IO(path, "a", background=bg)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            io.dump_snapshot(ps)
            t1 = time.perf_counter()
            io.flush()
            t2 = time.perf_counter()
            io.close()
            out["dump_" + tag] = {"call_ms": (t1 - t0) * 1e3, "complete_ms": (t2 - t0) * 1e3,
                                  "file_bytes": os.path.getsize(path)}
        t0 = time.perf_counter()
        back = IO(os.path.join(tmp, "sync.hdf5"), "r").load_snapshot()
        torch.cuda.synchronize()
        out["load_ms"] = (time.perf_counter() - t0) * 1e3
        out["load_bit_equal"] = all(torch.equal(getattr(back, k), getattr(ps, k))
                                    for k in ("id", "mass", "rx", "ry", "rz", "vx", "vy", "vz"))
        out["ms_per_step"] = {}
        for tag, bg in (("no dumpper", None), ("worldline sync", False), ("worldline background", True)):
            ps = ParticleSystem.from_arrays(**d)
            io = None if bg is None else IO(os.path.join(tmp, "wl_%s.hdf5" % tag.split()[-1]), "a",
                                            background=bg)
            kw = {} if io is None else {"dumpper": io, "dump_freq": 1}
            integ = Integrator(dt, 0.0, ps, method="sia21s.kdk", **kw)
            integ.evolve_step(dt)
            if io is not None:
                io.flush()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(steps):
                integ.evolve_step((k + 2) * dt)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            if io is not None:
                io.close()
            t2 = time.perf_counter()
            out["ms_per_step"][tag] = (t1 - t0) / steps * 1e3
            if io is not None:
                out["ms_per_step"][tag + ", writes drained"] = (t2 - t0) / steps * 1e3
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["precision", "adjoint", "binaries", "ensemble", "kernels",
                                            "integrators", "snapshots"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--reps", type=int, default=None, help="kernels: timed calls per kernel")
    ap.add_argument("--kernels", default=None, help="kernels: comma-separated kernel names")
    ap.add_argument("--precisions", default=None, help="kernels: comma-separated, ds32/ds32x/float64")
    ap.add_argument("--methods", default=None, help="integrators: comma-separated method names")
    args = ap.parse_args()
    kw = {}
    if args.steps:
        kw["steps"] = args.steps
    if args.n:
        kw["n"] = args.n
    for k in ("reps", "kernels", "precisions", "methods"):
        if getattr(args, k) is not None:
            kw[k] = getattr(args, k)
    fn = {"precision": precision_run, "adjoint": adjoint_run, "binaries": binaries_run,
          "ensemble": ensemble_run, "kernels": kernels_run, "integrators": integrators_run,
          "snapshots": snapshots_run}[args.which]
    from .clocks import Clocks
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    out = fn(**kw)
    out["clocks"] = clocks.stop()   # SM clock and throttle reasons over the whole run
    print(json.dumps(out, default=float))


if __name__ == "__main__":
    main()
