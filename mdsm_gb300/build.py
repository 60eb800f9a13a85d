"""In-tree build of libmdsm_gb300.so for sm_103a (nvcc, no cmake).

Every translation unit is compiled in parallel with one -gencode, then linked into
mdsm_gb300/_lib/libmdsm_gb300.so.  Host code is compiled with -ffp-contract=off: the DM shift
tables must be rounded operation by operation as the reference rounds them.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
# objects are kept per host architecture: a tree copied between machines never links stale ones
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(OUT_DIR, "libmdsm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "mdsm_gb300.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH,
           "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", CSRC,
           "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    stamp = os.path.join(BUILD, "lib.stamp")
    if (not os.path.exists(LIB) or not os.path.exists(stamp)
            or os.path.getmtime(stamp) < newest or os.path.getmtime(LIB) < newest):
        cmd = [nvcc(), "-shared", "-o", LIB, *objs, *ARCH, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        with open(stamp, "w") as f:
            f.write(LIB + "\n")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
