"""Build libtupan_gb300.so in-tree with nvcc for sm_103a.

    python -m tupan_gb300.build          # or tupan_gb300.build.build()

Compiles every translation unit in tupan_gb300/csrc in parallel (one
-gencode, -lineinfo) and links tupan_gb300/_lib/libtupan_gb300.so with the
CUDA runtime linked statically.  Objects go to tupan_gb300/_build/.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libtupan_gb300.so")
SOURCES = ("tg_api.cu", "tg_fp64.cu", "tg_ds32.cu", "tg_order.cu", "tg_probe.cu", "tg_noalloc.cu",
           "tg_integrate.cu", "tg_sia.cu")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            exe = cand
    if exe is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tupan_gb300")
    return exe


def flags(extra=()):
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-I" + os.path.join(os.path.dirname(HERE), "include")] + list(extra)


def build(force=False, extra=(), verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "tupan_gb300.h"))
    newest = max(os.path.getmtime(d) for d in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and not extra:
        return LIB
    exe = nvcc()
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [exe] + flags(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out))
    tmp = LIB + ".tmp"
    cmd = [exe, ARCH, "-shared", "-o", tmp] + objs
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n" + out.stdout + out.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
