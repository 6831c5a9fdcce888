"""Build libnmg.so (all CUDA kernels + the C ABI) for sm_103a, in-tree.

Each csrc/*.cu is compiled to an object in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then linked
into neural-mixture-guiding_gb300/_build/libnmg.so. Rebuilds only what is
older than its sources (any header change rebuilds everything).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnmg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    hdr_t = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    objs, jobs = [], []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_t):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (os.path.basename(src), r.stderr[-6000:]))
        os.replace(obj + ".tmp", obj)
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for err in ex.map(compile_one, jobs):
            if verbose and err.strip():
                print(err)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp.%d" % os.getpid()
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
