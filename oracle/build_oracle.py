"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so``: the C++ restatement in ``oracle.cpp``,
  compiled with g++ and OpenMP.  Runs on x86 and on Arm alike.
* ``oracle/_ref/ref_kernels.cubin``: the reference's own CUDA kernels
  (``tsqr_kernel``, ``tsgemm_tsqr``, ``gemm_blockqr``) compiled unmodified for
  sm_103a from the reference checkout, only when that checkout is present.  A
  cubin is device code, so it is built here once and loaded on any host by
  ``oracle/ref_launch.cpp`` through the CUDA driver API.
* ``oracle/_build/libref_launch.so``: that host-side launcher (our code; it
  restates the reference host schedule and needs no reference source).
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: TSQR_REFERENCE_SRC, or --ref-src on the command
# line, else the checkout's location in the build container.
REF_SRC_DEFAULT = os.environ.get("TSQR_REFERENCE_SRC", "/root/reference")


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    out = os.path.join(BUILD, "liboracle.so")
    if force or _newer(out, [src]):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def _nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", shutil.which("nvcc") or ""):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def build_ref_cubin(ref_src=REF_SRC_DEFAULT, force=False):
    """Compile the reference kernels, unmodified, into one sm_103a cubin.

    The translation unit is ``oracle/ref_kernels_tu.cu``, which only includes
    the reference headers (so the explicit template instantiations at
    TallShinnyQR.h:75-84, block_QR.h:61-70, kernelQR.h:498-507 are emitted).
    ``-DmemoryClockRate=memoryBusWidth`` lets utils.h:114 compile under CUDA 13,
    where that cudaDeviceProp field is gone; it touches only a host diagnostic.
    Returns the cubin path, or None when the reference checkout is absent.
    """
    if not os.path.isdir(ref_src):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    tu = os.path.join(HERE, "ref_kernels_tu.cu")
    out = os.path.join(REF_OUT, "ref_kernels.cubin")
    deps = [tu] + [os.path.join(ref_src, f) for f in ("kernelQR.h", "TallShinnyQR.h", "block_QR.h", "utils.h")]
    if force or _newer(out, deps):
        _run([_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3",
              "-DmemoryClockRate=memoryBusWidth", "-I", ref_src, tu, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_ref_launcher(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_launch.cpp")
    out = os.path.join(BUILD, "libref_launch.so")
    if force or _newer(out, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-I/usr/local/cuda/include",
              "-o", out + ".tmp", "-ldl"])
        os.replace(out + ".tmp", out)
    return out


def build_all(force=False, ref_src=None):
    paths = {"oracle": build_oracle(force)}
    paths["ref_cubin"] = build_ref_cubin(ref_src or REF_SRC_DEFAULT, force=force)
    paths["ref_launch"] = build_ref_launcher(force)
    return paths


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ref-src", default=None, help="the reference checkout (default: TSQR_REFERENCE_SRC or "
                                                    "the build container's checkout)")
    a = ap.parse_args()
    print(build_all(force=a.force, ref_src=a.ref_src))
