"""Build libgbba.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each .cu file under csrc/ is compiled in parallel with nvcc, then linked into
one shared library with the CUDA runtime linked statically, so that the
library loads without any Python or torch dependency.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbba.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def flags(extra=()):
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I" + os.path.join(HERE, "..", "include"), *extra]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def build(verbose=False, ptxas_info=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(HERE, "..", "include", f) for f in os.listdir(os.path.join(HERE, "..", "include"))]
    objs, cmds = [], []
    for src in sources():
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, hdrs) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            cmds.append([cc, *flags(extra), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(run, cmds):
            logs.append(out)
    relink = cmds or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if relink:
        tmp = LIB + ".tmp"
        run([cc, ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    if verbose:
        for line in logs:
            sys.stderr.write(line)
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(verbose=True, ptxas_info="-v" in sys.argv)
    print(lib)
