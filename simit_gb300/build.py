"""Build libsimit_gb300.so in-tree with nvcc for sm_103a (no cmake).

Each .cu / .cpp under csrc/ is compiled in parallel into _build/, then linked
with -shared.  Files named *_exact.cu are compiled with --fmad=false so their
FP arithmetic follows the reference's unfused operation order.
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libsimit_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    return "nvcc"


def _sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or (f.endswith(".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _deps_mtime():
    m = 0.0
    for root in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(root):
            if f.endswith((".cuh", ".h", ".hpp")):
                m = max(m, os.path.getmtime(os.path.join(root, f)))
    return m


def _compile(src, hdr_mtime, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj, None
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-I", os.path.dirname(HERE), "-c", src, "-o", obj]
    if src.endswith("_exact.cu"):
        cmd.insert(1, "--fmad=false")
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None, "%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, (r.stderr if verbose else None)


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hm = _deps_mtime()
    objs, errs = [], []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for obj, msg in ex.map(lambda s: _compile(s, hm, verbose), srcs):
            if obj is None:
                errs.append(msg)
            else:
                objs.append(obj)
                if msg:
                    print(msg, file=sys.stderr)
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    newest = max(os.path.getmtime(o) for o in objs)
    stamp = os.path.join(BUILD, "lib.stamp")
    if (not os.path.exists(LIB) or not os.path.exists(stamp)
            or os.path.getmtime(LIB) < newest):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl"]
        subprocess.check_call(cmd)
        open(stamp, "w").write(platform.machine())
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
