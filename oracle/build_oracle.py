"""Build the CPU oracle (test infrastructure) into oracle/_build/libnmg_oracle.so.

The oracle is plain C++ (g++, OpenMP). It is compiled with
-ffp-contract=off so that x86-64 and aarch64 hosts evaluate the FP32
restatement with the same operation sequence (no fused multiply-adds).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnmg_oracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
HEADERS = [os.path.join(HERE, "nmg_oracle.hpp")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in SOURCES + HEADERS)


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_reference():
    """Compile the reference's own code for the oracle (only where its checkout exists: build_ref.sh
    looks for it, at $NMG_REFERENCE when that is set)."""
    script = os.path.join(HERE, "build_ref.sh")
    if subprocess.run(["bash", script, "--check"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode:
        return None
    out = os.path.join(HERE, "_ref", "libnmgref.so")
    srcs = [os.path.join(HERE, f) for f in ("ref_shim.cu", "ref_tcnn_kernels.cu", "ref_tcnn_layout.cu",
                                            "tcnn_host_headers.py")] + [script]
    if os.path.exists(out) and all(os.path.getmtime(p) <= os.path.getmtime(out) for p in srcs):
        return out
    r = subprocess.run(["bash", script], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build_ref.sh failed:\n" + r.stderr[-4000:])
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    if "--ref" in sys.argv:
        print(build_reference())
