"""Benchmark: Gint/s of the split-FP32 Acc and AccJerk kernels on one GB300.

Workload (the precision-form configuration): a Plummer sphere of N = 65536
particles with a Salpeter mass function (slope -2.35, masses in [0.1, 100],
total mass 1), pair softening eps2 = 1e-6 (eps = 1e-3), Henon units, seeded
synthetic inputs.  One step = one Acc and one AccJerk evaluation of all N
i-particles against all N j-particles in split FP32 (2 N^2 interactions).

Printed JSON line (rank 0):
  value        interactions / second over the timed steps, inputs resident in
               HBM (device pointers through the C ABI), Gint/s
  e2e          the same metric through the drop-in host entry points
               acc_kernel / acc_jerk_kernel (libtupan.h signatures) with host
               buffers, host<->device copies inside the timed region
  roofline     the AccJerk pairwise kernel (ds32_ord<AccJerkOrd>):
               reference-counted 42 flop/interaction x interactions / that
               kernel's own duration (CUDA events the library records around
               it on the call's stream, tg_time_pair_kernel), against the FP32
               FMA peak measured on this GPU by tg_probe_fma_tflops; call_frac
               is the same over the whole call (spatial sort, record
               preparation, plan, pairwise kernel, double-single recompute)
  fp64         the FP64 GPU kernels on the same workload (bit-identical to the
               reference C backend) and the split-FP32 speed-up over them
  force_error  per-particle |a_ds32 - a_fp64| / |a_fp64| (and jerk)
  other_kernels  split-FP32 Phi, SnapCrackle, Tstep and PNAcc on the same
               workload, FP64 Sakura on its first 4096 particles (device time)
  energy       |dE/E| of a short shared-step SIA21 kdk leapfrog of the same
               workload in split FP32 and in FP64, and their ratio
  cpu_baseline the reference's own C backend (compiled unmodified from the
               installed copy into oracle/_ref by __graft_entry__.build; kind
               "reference"), else the CPU oracle port (same algorithm and
               operation order; kind "port"), on all host cores, bounded sample
  clocks       nvidia-smi SM clock and throttle reasons during the timed region

`--impl reference` times that same CPU implementation on a bounded sample of
the same workload and prints the same metric; it imports nothing of the
GPU library.
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_DEFAULT = 65536
EPS = 1e-3
SEED = 20261203
FLOP_ACC = 20       # tupan/lib/src/acc_kernel_common.h:38
FLOP_ACC_JERK = 42  # tupan/lib/src/acc_jerk_kernel_common.h:56
# DRAM bytes (read + write) of one AccJerk pairwise-kernel launch on this
# workload, from an ncu capture (profiles/ds32_ord_acc_jerk_n65536.txt)
TRAFFIC_ACC_JERK_N65536 = 7.35e6
METRIC = "Gint/s Acc+AccJerk split-FP32 (N=65536 Plummer-Salpeter, eps2=1e-6)"
# library kernels per ordered Acc or AccJerk call: spatial order (bounds,
# keys, the radix sort's histogram, exclusive-sum and four one-sweep passes),
# record preparation, i-tile boxes, plan, the prefix sum's two launches, CTA
# bounds, the pairwise kernel and the double-single recompute
LAUNCHES_PER_CALL = 17
LAUNCHES_PER_STEP = 2 * LAUNCHES_PER_CALL
SMALL_SIZES = (4096, 16384)
P5 = ("mass", "rx", "ry", "rz", "eps2")
P8 = P5 + ("vx", "vy", "vz")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--particles", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=3.0,
                    help="target wall time of each CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--energy-steps", type=int, default=8,
                    help="steps of the leapfrog whose |dE/E| is reported in both precisions")
    return ap.parse_args()


def workload(n, rank):
    from tupan_gb300.ics import Salpeter, plummer_arrays
    return plummer_arrays(n, EPS, imf=Salpeter(0.1, 100.0), seed=SEED + rank)


def config(n):
    return {"workload": "plummer-salpeter", "n": n, "imf": "salpeter -2.35 [0.1,100], M=1",
            "eps2_pair": 2 * (EPS * EPS / 2), "units": "henon", "step": "acc + acc_jerk, i=j=all",
            "interactions_per_step": 2 * n * n,
            "precision": "ds32 (hi/lo or block-relative positions, Kahan-folded FP32 sums, "
                         "double-single recompute of strongly cancelling particles)",
            "l2": "flushed between timed steps (256 MiB write)", "seed": SEED}


def pn_flop(order):
    """Flop per PNAcc interaction: the reference's 40 for the pair geometry
    (pnacc_kernel_common.h:70, "40+???") plus the generated post-Newtonian
    polynomial up to `order` (tupan_gb300/csrc/tg_pn_terms.cuh: powers, then
    one block per order; fma = 2, every other +, -, * = 1)."""
    import re
    src = open(os.path.join(ROOT, "tupan_gb300", "csrc", "tg_pn_terms.cuh")).read()
    body = src[src.index("pn_factors"):]
    body = body[body.index("{") + 1:]
    total, cur = 0, None
    for line in body.splitlines():
        m = re.search(r"if \(order >= (\d)ul\)", line)
        if m:
            cur = int(m.group(1))
            continue
        code = line.split("//")[0].strip()
        if not code.endswith(";") or code.startswith(("return", "if")) or (cur is not None and cur > order):
            continue
        f = 2 * code.count("fma(")
        t = re.sub(r"T\(-?[\d.]+\)", "K", code).replace("fma(", "(")
        if "+=" in t or "-=" in t:
            f += 1
        t = t.replace("+=", "=").replace("-=", "=")
        rhs = t.split("=", 1)[1] if "=" in t else ""
        f += len(re.findall(r"[\*\+]|(?<=[\w\)])\s*-", rhs))
        total += f
    return 40 + total


# ---------------------------------------------------------------------------
# CPU baseline (oracle port of the reference algorithm)
# ---------------------------------------------------------------------------
def cpu_impl():
    """The reference's own C backend when oracle/_ref holds its build, else
    the oracle port: (calc(name, I, J, threads), kind)."""
    from oracle import oracle as om
    if om.reference_available():
        ref = om.ReferenceLib()
        from concurrent.futures import ThreadPoolExecutor

        def calc(name, I, J, threads):
            # the reference C is single-threaded: contiguous i-slices on a
            # thread pool (ctypes releases the GIL during the call)
            ni = len(I["mass"])
            cuts = np.linspace(0, ni, threads + 1).astype(int)
            with ThreadPoolExecutor(threads) as ex:
                list(ex.map(lambda k: ref.calc(name, {f: v[cuts[k]:cuts[k + 1]] for f, v in I.items()}, J),
                            [k for k in range(threads) if cuts[k + 1] > cuts[k]]))
        return calc, "reference"
    om.build()
    orc = om.Oracle()
    return (lambda name, I, J, threads: orc.calc(name, I, J, nthreads=threads)), "port"


def cpu_sample(d, seconds, threads):
    """Time FP64 Acc + AccJerk of the first ni_s i-particles against all N.

    ni_s is calibrated so one sample takes about `seconds` of wall time."""
    calc, kind = cpu_impl()
    n = len(d["mass"])

    def run(ni):
        I = {k: v[:ni] for k, v in d.items()}
        t0 = time.perf_counter()
        calc("acc", I, d, threads)
        calc("acc_jerk", I, d, threads)
        return time.perf_counter() - t0

    ni = max(threads, 64)
    t = run(ni)
    while t < 0.2 and ni < n:
        ni = min(n, ni * 4)
        t = run(ni)
    ni = int(min(n, max(threads, ni * seconds / max(t, 1e-6))))
    t = run(ni)
    return {"value": 2.0 * ni * n / t / 1e9, "unit": "Gint/s", "cores": threads,
            "kind": kind, "seconds": t,
            "sample": "FP64 acc + acc_jerk, %d i-particles x %d j-particles (%.3g interactions)"
                      % (ni, n, 2.0 * ni * n)}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    d = workload(args.particles, 0)
    threads = os.cpu_count() or 1
    for _ in range(max(args.warmup, 0)):
        cpu_sample(d, min(args.cpu_seconds, 1.0), threads)
    vals = [cpu_sample(d, args.cpu_seconds, threads) for _ in range(max(args.steps, 1))]
    v = float(np.median([x["value"] for x in vals]))
    secs = sum(x["seconds"] for x in vals)
    base = dict(vals[0])
    base["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gint/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / len(vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(args.particles), "cpu_baseline": base,
            "e2e": {"value": v, "unit": "Gint/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def rel_errors(got, want):
    d = np.sqrt(((got - want) ** 2).sum(0))
    n = np.sqrt((want ** 2).sum(0))
    r = d[n > 0] / n[n > 0]
    return {"max": float(r.max()), "p99": float(np.percentile(r, 99)),
            "median": float(np.median(r)), "rms": float(np.sqrt((r * r).mean()))}


def small_sizes(dev, sp):
    """Acc and AccJerk at N = 4096 and 16384 (same workload family): median
    CUDA-event time of 21 split FP32 and 21 FP64 calls (after one untimed
    call) and the split-FP32 force error against FP64."""
    import torch
    from tupan_gb300 import _native
    out = {}
    for n in SMALL_SIZES:
        d = workload(n, 0)
        T = {k: torch.tensor(d[k], dtype=torch.float64, device=dev) for k in P8}
        rec = {}
        res = {}
        for name, fields, no in (("acc", P5, 3), ("acc_jerk", P8, 6)):
            for prec, pname, reps in ((_native.PREC_DS32, "ds32", 21), (_native.PREC_FP64, "fp64", 21)):
                o = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(no)]

                def call():
                    _native.call_device(name, n, [T[k].data_ptr() for k in fields], n,
                                        [T[k].data_ptr() for k in fields], (), [x.data_ptr() for x in o], prec, sp)
                call()
                ms = []
                for _ in range(reps):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    call()
                    e1.record()
                    e1.synchronize()
                    ms.append(e0.elapsed_time(e1))
                med = float(np.median(ms))
                rec["%s_%s" % (name, pname)] = {"ms": med, "gint_s": n * n / (med * 1e-3) / 1e9}
                res[(name, pname)] = np.stack([x.cpu().numpy() for x in o])
        rec["force_error_acc_max"] = rel_errors(res[("acc", "ds32")], res[("acc", "fp64")])["max"]
        rec["force_error_jerk_max"] = rel_errors(res[("acc_jerk", "ds32")][3:], res[("acc_jerk", "fp64")][3:])["max"]
        out[str(n)] = rec
    return out


# reference flop counts per interaction (<kernel>_kernel_common.h)
FLOP_OTHER = {"phi": 14, "snap_crackle": 114, "tstep": 42}


def other_kernels(dev, sp, T, outs, n, peak32):
    """The other hot-path kernels on the same workload: split-FP32 Phi,
    SnapCrackle (a, j from the split-FP32 AccJerk above), Tstep (eta 1/1024)
    and PNAcc (order 5, c = 1e4) at N = n, and FP64 Sakura (flag -1,
    dt = 1/1024) on the workload's first 4096 particles: median CUDA-event
    time of 5 calls after one untimed call."""
    import torch
    from tupan_gb300 import _native
    T = dict(T)
    for k, x in zip(("ax", "ay", "az", "jx", "jy", "jz"), outs[3:9]):
        T[k] = x
    c = 1e4
    pn = (5,) + tuple(c ** -k for k in range(1, 8))
    jobs = [("phi", n, _native.PREC_DS32, ()), ("snap_crackle", n, _native.PREC_DS32, ()),
            ("tstep", n, _native.PREC_DS32, (1.0 / 1024,)), ("pnacc", n, _native.PREC_DS32, pn),
            ("sakura", 4096, _native.PREC_FP64, (1.0 / 1024, -1))]
    res = {}
    for name, m, prec, sc in jobs:
        fields, _, names = _native.SPECS[name]
        ptrs = [T[k].data_ptr() for k in fields]
        o = [torch.empty(m, dtype=torch.float64, device=dev) for _ in names]

        def call():
            _native.call_device(name, m, ptrs, m, ptrs, sc, [x.data_ptr() for x in o], prec, sp)
        call()
        ms = []
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        med = float(np.median(ms))
        rec = {"n": m, "precision": "ds32" if prec == _native.PREC_DS32 else "fp64", "ms": med,
               "gint_s": m * m / (med * 1e-3) / 1e9}
        flop = FLOP_OTHER.get(name) or (pn_flop(5) if name == "pnacc" else None)
        if flop and peak32 > 0:
            rec["flop_per_interaction"] = flop
            rec["frac"] = flop * m * m / (med * 1e-3) / 1e12 / peak32
        res[name] = rec
    st = _native.sync_status(sp)
    res["status"] = st
    return res


def energy_drift(n, steps):
    """|dE/E| of a shared-step SIA21 kdk leapfrog (dt = 1/1024, Tstep each
    step) of the benchmark workload, split FP32 against FP64; energies from
    the FP64 Phi kernel (tupan_gb300.runs.precision_run)."""
    from tupan_gb300.runs import precision_run
    r = precision_run(n=n, steps=steps, dt=1.0 / 1024, seed=SEED, probe_every=0)
    return {"steps": steps, "dt": 1.0 / 1024, "method": "sia21s.kdk",
            "ds32": r["ds32"]["rel_energy_error"], "fp64": r["float64"]["rel_energy_error"],
            "ratio_ds32_over_fp64": r["energy_drift_ratio_ds32_over_fp64"],
            "ms_per_step_ds32": r["ds32"]["ms_per_step"], "ms_per_step_fp64": r["float64"]["ms_per_step"]}


def ours(args, rank, world, dist):
    import torch
    from tupan_gb300 import _native

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = args.particles
    d = workload(n, rank)
    T = {k: torch.tensor(d[k], dtype=torch.float64, device=dev) for k in P8}
    outs = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(9)]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    ptr = lambda keys: [T[k].data_ptr() for k in keys]

    def acc(prec, o):
        _native.call_device("acc", n, ptr(P5), n, ptr(P5), (), [x.data_ptr() for x in o], prec, sp)

    def acc_jerk(prec, o):
        _native.call_device("acc_jerk", n, ptr(P8), n, ptr(P8), (), [x.data_ptr() for x in o], prec, sp)

    DS = _native.PREC_DS32
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    from tupan_gb300.clocks import Clocks
    clocks = Clocks(dev.index)
    clocks.start()
    # warm-up: W steps, and at least one second of load so clocks settle
    t_end = time.perf_counter() + 1.0
    w = 0
    while w < max(args.warmup, 0) or time.perf_counter() < t_end:
        acc(DS, outs[:3])
        acc_jerk(DS, outs[3:])
        torch.cuda.synchronize()
        w += 1

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    _native.pair_kernel_time(_native.KERNEL_ACC)        # drop earlier records
    _native.pair_kernel_time(_native.KERNEL_ACC_JERK)
    _native.lib.tg_time_pair_kernel(1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    torch.cuda.nvtx.range_push("bench_timed")   # ncu --nvtx-include bench_timed/
    for s in range(args.steps):
        flush.zero_()
        ev[s][0].record(stream)
        acc(DS, outs[:3])
        ev[s][1].record(stream)
        acc_jerk(DS, outs[3:])
        ev[s][2].record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    _native.lib.tg_time_pair_kernel(0)
    k_acc_ms, k_acc_n = _native.pair_kernel_time(_native.KERNEL_ACC)
    k_aj_ms, k_aj_n = _native.pair_kernel_time(_native.KERNEL_ACC_JERK)
    if n >= 4096 and (k_acc_n != args.steps or k_aj_n != args.steps):
        # every timed call at these sizes takes the ordered path
        raise RuntimeError("pairwise-kernel events: %d Acc and %d AccJerk launches recorded for %d steps"
                           % (k_acc_n, k_aj_n, args.steps))
    if dist:
        dist.barrier()
    clk = clocks.stop()
    st = _native.sync_status(sp)
    if st:
        raise RuntimeError("kernel status bits set: %d" % st)
    t_acc = [ev[s][0].elapsed_time(ev[s][1]) for s in range(args.steps)]
    t_aj = [ev[s][1].elapsed_time(ev[s][2]) for s in range(args.steps)]
    step_ms = float(np.sum(t_acc) + np.sum(t_aj)) / args.steps
    if dist:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    inter = 2.0 * n * n
    value = world * inter / (step_ms * 1e-3) / 1e9
    aj_ms = float(np.median(t_aj))
    acc_ms = float(np.median(t_acc))

    ds_acc = np.stack([x.cpu().numpy() for x in outs[:3]])
    ds_aj = np.stack([x.cpu().numpy() for x in outs[3:]])

    peak32 = _native.lib.tg_probe_fma_tflops(0, 20000, sp)
    peak64 = _native.lib.tg_probe_fma_tflops(1, 2000, sp)
    # the pairwise kernel's own average duration (events around its launch)
    kaj_ms = k_aj_ms / k_aj_n if k_aj_n else aj_ms
    kacc_ms = k_acc_ms / k_acc_n if k_acc_n else acc_ms
    achieved = FLOP_ACC_JERK * n * n / (kaj_ms * 1e-3) / 1e12
    call_achieved = FLOP_ACC_JERK * n * n / (aj_ms * 1e-3) / 1e12
    line = {"metric": METRIC, "value": value, "unit": "Gint/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "ds32", "data": "synthetic",
            "config": config(n), "gpu_launches": LAUNCHES_PER_STEP * args.steps,
            "kernels": {"acc_ds32": {"ms": acc_ms, "gint_s": n * n / (acc_ms * 1e-3) / 1e9,
                                     "pair_kernel_ms": kacc_ms, "pair_kernel_launches": k_acc_n},
                        "acc_jerk_ds32": {"ms": aj_ms, "gint_s": n * n / (aj_ms * 1e-3) / 1e9,
                                          "pair_kernel_ms": kaj_ms, "pair_kernel_launches": k_aj_n}},
            "roofline": {"bound": "fp32", "kernel": "ds32_ord<AccJerkOrd<2>>",
                         "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                         "frac": achieved / peak32 if peak32 > 0 else None,
                         "call_achieved": call_achieved,
                         "call_frac": call_achieved / peak32 if peak32 > 0 else None,
                         "traffic": TRAFFIC_ACC_JERK_N65536 if n == N_DEFAULT else None,
                         "traffic_source": "ncu dram__bytes_read+write of one AccJerk launch at N=65536",
                         "flop_per_interaction": FLOP_ACC_JERK,
                         "peak_source": "measured: tg_probe_fma_tflops (FFMA2 chains, this GPU)",
                         "peak_fp64_tflops": peak64,
                         # the FP32 issue-rate view of the same kernel: pipe
                         # utilisation from its ncu capture (a profile of
                         # this kernel and workload, not of this run)
                         "issue_rate_ncu": {"sm__pipe_fma_cycles_active": 0.782,
                                            "sm__pipe_xu_cycles_active": 0.247,
                                            "source": "profiles/ds32_ord_acc_jerk_n65536.txt"},
                         "acc_frac": (FLOP_ACC * n * n / (kacc_ms * 1e-3) / 1e12) / peak32 if peak32 > 0 else None},
            "clocks": clk, "wall_s": wall}

    if not args.no_fp64:
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        f_out = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(9)]
        e[0].record(stream)
        acc(_native.PREC_FP64, f_out[:3])
        e[1].record(stream)
        acc_jerk(_native.PREC_FP64, f_out[3:])
        e[2].record(stream)
        torch.cuda.synchronize()
        f_acc_ms, f_aj_ms = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        f_acc = np.stack([x.cpu().numpy() for x in f_out[:3]])
        f_aj = np.stack([x.cpu().numpy() for x in f_out[3:]])
        fp64_v = inter / ((f_acc_ms + f_aj_ms) * 1e-3) / 1e9
        line["fp64"] = {"acc_ms": f_acc_ms, "acc_jerk_ms": f_aj_ms, "value": fp64_v, "unit": "Gint/s",
                        "acc_jerk_gint_s": n * n / (f_aj_ms * 1e-3) / 1e9,
                        "ds32_speedup": value / world / fp64_v,
                        "acc_jerk_ds32_speedup": f_aj_ms / aj_ms}
        line["force_error"] = {"acc": rel_errors(ds_acc, f_acc), "acc_in_acc_jerk": rel_errors(ds_aj[:3], f_aj[:3]),
                               "jerk": rel_errors(ds_aj[3:], f_aj[3:]),
                               "against": "FP64 GPU kernels (bit-identical to the reference C backend)"}

    # ---- the smaller sizes of the same workload (parity/measurement only) --
    if rank == 0 and not args.no_fp64:
        line["sizes"] = small_sizes(dev, sp)
        line["other_kernels"] = other_kernels(dev, sp, T, outs, n, peak32)
        line["energy"] = energy_drift(n, args.energy_steps)

    # ---- end to end through the drop-in host entry points ---------------
    pin = {k: torch.tensor(d[k], dtype=torch.float64).pin_memory() for k in P8}
    hp = {k: ctypes.c_void_p(v.data_ptr()) for k, v in pin.items()}
    hout = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(9)]
    ho = [ctypes.c_void_p(x.data_ptr()) for x in hout]
    _native.lib.tg_set_host_precision(DS)

    def e2e_step():
        _native.lib.acc_kernel(n, *[hp[k] for k in P5], n, *[hp[k] for k in P5], *ho[:3])
        _native.lib.acc_jerk_kernel(n, *[hp[k] for k in P8], n, *[hp[k] for k in P8], *ho[3:])

    e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    _native.lib.tg_set_host_precision(_native.PREC_FP64)
    line["e2e"] = {"value": world * inter / e2e_s / 1e9, "unit": "Gint/s",
                   # i- and j-sets are the same host arrays: each is copied once
                   "h2d_bytes_per_step": 8 * n * (5 + 8), "d2h_bytes_per_step": 8 * n * (3 + 6),
                   "ms_per_step": e2e_s * 1e3,
                   "path": "acc_kernel + acc_jerk_kernel (libtupan.h signatures), pinned host buffers"}
    if rank == 0:
        line["cpu_baseline"] = cpu_sample(d, args.cpu_seconds, os.cpu_count() or 1)
        one = cpu_sample(d, min(args.cpu_seconds, 2.0), 1)
        line["cpu_baseline"]["single_core"] = {"value": one["value"], "unit": one["unit"],
                                               "sample": one["sample"]}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        backend = "nccl" if (args.impl == "ours" and torch.cuda.is_available()) else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        tdist.init_process_group(backend)
        dist = tdist
    try:
        if args.impl == "reference":
            reference_arm(args, rank, world)
        else:
            ours(args, rank, world, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
