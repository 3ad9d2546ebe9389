"""Builds libflou_cuda.so in-tree for sm_103a (no cmake).

Each translation unit under csrc/ is compiled by its own nvcc process (in parallel), then
linked into lib/libflou_cuda.so.  Sources are recompiled only when they or a header changed.
`build(checked=True)` (or `python build.py --checked`) builds lib/libflou_cuda_checked.so with
-DFLOU_CUDA_CHECKED: every kernel checks its computed indices against the array sizes and
reports an out-of-range one through the status word (FLOU_ERR_INDEX) instead of accessing it.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libflou_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, extra, objdir=OBJ):
    obj = os.path.join(objdir, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return obj, None
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, "compile failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr)
    return obj, None


def _weight(src):
    """Rough compile cost of a translation unit, so that the slowest start first."""
    name = os.path.basename(src)
    for prefix, w in (("adjoint_hybrid", 4), ("adjoint_split", 3), ("elem_", 2), ("batch", 2), ("adjoint", 1)):
        if name.startswith(prefix):
            return w
    return 0


def build_set(variants, verbose=False):
    """Builds one library per (extra flags, checked) variant, compiling every variant's
    translation units in one worker pool, slowest first; returns the library paths."""
    plans = []
    for extra, checked in variants:
        objdir = os.path.join(OBJ, "checked") if checked else OBJ
        lib = os.path.join(LIBDIR, "libflou_cuda_checked.so") if checked else LIB
        flags = list(extra) + (["-DFLOU_CUDA_CHECKED"] if checked else [])
        os.makedirs(objdir, exist_ok=True)
        plans.append((objdir, lib, flags))
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = sorted(((k, s) for k in range(len(plans)) for s in srcs), key=lambda j: -_weight(j[1]))
    workers = min(len(jobs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        results = list(ex.map(lambda j: _compile(j[1], plans[j[0]][2], plans[j[0]][0]), jobs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("\n".join(errs))
    libs = []
    for k, (objdir, lib, _) in enumerate(plans):
        objs = sorted(o for (kk, _), (o, _) in zip(jobs, results) if kk == k)
        if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
            cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
        if verbose:
            print("built", lib)
        libs.append(lib)
    return libs


def build(verbose=False, extra=(), checked=False):
    return build_set([(extra, checked)], verbose)[0]


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--checked"]
    build(verbose=True, extra=args, checked="--checked" in sys.argv[1:])
