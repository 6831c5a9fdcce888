"""Host-callable copies of tiny-cuda-nn's kernel headers (TEST INFRASTRUCTURE ONLY).

    python oracle/tcnn_host_headers.py <tcnn include dir> <output include dir>

oracle/build_ref.sh runs this while it builds oracle/_ref/ from the
reference checkout; the copies live only under oracle/_ref/build/ and are
never committed. They let oracle/ref_tcnn_kernels.cu run the reference's own
encoding and optimiser kernels on the host, once per thread index, to write
golden vectors. The arithmetic of every function is left as it is; three
mechanical edits make it callable from host code:
  * each header is cut before its first class template (the Encoding /
    Optimizer classes, whose kernel launches and device lambdas cannot be
    host code), keeping the includes, the device helpers and the kernels,
    and the namespace is closed again;
  * function qualifiers `__device__` become `__host__ __device__` (device
    lambdas, `] __device__ (`, and functions already `__host__ __device__`
    are left alone);
  * `__global__` becomes `__host__`, so a kernel is an ordinary function whose
    thread-index built-ins the including file maps to host variables.
common_device.h gets only the qualifier edit (it has no classes or kernels).
"""
import os
import re
import sys

KERNEL_HEADERS = ["encodings/grid.h", "encodings/spherical_harmonics.h", "encodings/oneblob.h",
                  "optimizers/adam.h", "optimizers/ema.h"]


def widen(text):
    text = text.replace("__host__ __device__", "\x00HD\x00")
    text = re.sub(r"\]\s*__device__\s*\(", lambda m: m.group(0).replace("__device__", "\x00LD\x00"), text)
    text = re.sub(r"\b__device__\b", "__host__ __device__", text)
    text = text.replace("\x00HD\x00", "__host__ __device__").replace("\x00LD\x00", "__device__")
    return text


def cut_before_class(text, path):
    lines = text.split("\n")
    for i in range(1, len(lines)):
        if lines[i].startswith("class ") and lines[i - 1].startswith("template <"):
            return "\n".join(lines[:i - 1]) + "\n\nTCNN_NAMESPACE_END\n"
    raise SystemExit("no class template found in %s" % path)


def main(src, dst):
    for rel in KERNEL_HEADERS:
        text = open(os.path.join(src, "tiny-cuda-nn", rel)).read()
        out = cut_before_class(text, rel)
        out = widen(out).replace("__global__", "__host__")
        path = os.path.join(dst, "tiny-cuda-nn", rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            fh.write(out)
    text = open(os.path.join(src, "tiny-cuda-nn", "common_device.h")).read()
    with open(os.path.join(dst, "tiny-cuda-nn", "common_device.h"), "w") as fh:
        fh.write(widen(text))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
