"""Register spills of the library's kernels, from ptxas's own report.

The build compiles every unit with `-Xptxas -warn-spills` and keeps the
report in tsqr_gb300/_build/<unit>.ptxas.log.  A kernel that spills reads and
writes local memory inside its loops, so a new or larger spill is a
performance regression: none of the kernels on the FP32 n <= 32 path may
spill, and the known spills below may not grow.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tsqr_gb300", "_build")

# kernel -> (spill store bytes, spill load bytes) at most
KNOWN = {
    # FP64 tile factor: 3 CTAs per SM cap it at 85 registers; the FP64 pipe
    # bounds this kernel
    "tsqr::factor_split_tiles<double, 32, 4, 8, 3, false>": (788, 1312),
    # the 64-column tile holds 128 values per thread
    "tsqr::factor_split_tiles<float, 64, 8, 16, 1, false>": (92, 92),
    "tsqr::factor_split_tiles<float, 64, 8, 8, 1, false>": (44, 44),
    "tsqr::factor_split_tiles<float, 64, 8, 4, 1, false>": (4, 4),
    "tsqr::factor_split_tiles<float, 64, 8, 2, 1, false>": (4, 4),
    # the precision form's fp64_scalars option: FP64 norm, beta and tau take
    # register pairs on the owner's chain (an option, off by default)
    "tsqr::factor_split_tiles<float, 16, 4, 16, 4, true>": (112, 248),
    "tsqr::factor_split_tiles<float, 32, 4, 16, 2, true>": (112, 248),
    "tsqr::factor_split_tiles<float, 64, 8, 16, 1, true>": (160, 160),
    "tsqr::factor_split_tiles<float, 64, 8, 8, 1, true>": (68, 68),
    "tsqr::factor_split_tiles<float, 64, 8, 4, 1, true>": (4, 4),
    "tsqr::factor_split_tiles<float, 64, 8, 2, 1, true>": (4, 4),
    # the TMA-staged tile factor: 8 bytes (two registers) of its loop state
    # at the 128-register limit of 2 CTAs per SM; measured at parity with the
    # register-load kernel on the level it serves
    "tsqr::factor_split_tiles_tma<float, 32, 4, 16, 2>": (8, 8),
    "tsqr::factor_split_tiles_tma<float, 16, 4, 16, 4>": (8, 8),
    # batched kernels: per-problem descriptors cost registers
    "tsqr::batched_apply<64, 256, 2, 1>": (88, 128),
    "tsqr::batched_apply<32, 256, 2, 2>": (80, 112),
    "tsqr::batched_factor_split<64, 8, 16, 1>": (4, 32),
    "tsqr::batched_factor_split<32, 4, 16, 2>": (16, 20),
    "tsqr::batched_factor_split<16, 4, 16, 4>": (12, 36),
    "tsqr::apply_qt_tiles<double, 64>": (32, 40),
    "tsqr::gram_partial_kernel<float>": (4, 4),
    "tsqr::gram_partial_kernel<double>": (4, 4),
}

WARN = re.compile(r"Registers are spilled to local memory in function '([^']+)', (\d+) bytes spill stores, "
                  r"(\d+) bytes spill loads")


def _demangle(names):
    out = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True, check=True)
    return out.stdout.splitlines()


def _kernel(name):
    name = name.replace("(anonymous namespace)::", "")
    if name.startswith("void "):
        name = name[5:]
    return name.split("(")[0]


@pytest.fixture(scope="module")
def spills(tg):
    if shutil.which("c++filt") is None:
        pytest.skip("c++filt not available")
    from tsqr_gb300 import build as tb
    logs = [os.path.join(BUILD, s.replace(".cu", ".ptxas.log")) for s in tb.SOURCES]
    if not all(os.path.exists(p) for p in logs):
        tb.build_lib(force=True)  # a library built before the reports were kept
    found = []
    for p in logs:
        with open(p) as f:
            found += WARN.findall(f.read())
    names = _demangle([f[0] for f in found]) if found else []
    return {_kernel(n): (int(f[1]), int(f[2])) for n, f in zip(names, found)}


def test_spill_report_is_on():
    from tsqr_gb300 import build as tb
    assert "-warn-spills" in tb.NVFLAGS


def test_no_new_or_larger_spills(spills):
    bad = {}
    for k, (st, ld) in spills.items():
        if k.startswith("__cuda_"):
            continue  # the CUDA math library's own slow paths (FP64 division and square root)
        lim = KNOWN.get(k)
        if lim is None or st > lim[0] or ld > lim[1]:
            bad[k] = (st, ld, lim)
    assert not bad, bad


@pytest.mark.parametrize("kernel", ["tsqr::factor_split_tiles<float, 32, 4, 16, 2, false>",
                                    "tsqr::factor_split_tiles<float, 16, 4, 16, 4, false>",
                                    "tsqr::apply_tiles<float, 32, 256, 2, 2>",
                                    "tsqr::tc_apply_tiles<32, 512, true>",
                                    "tsqr::tc_apply_tiles<64, 512, true>",
                                    "tsqr::gemm_tn_tma",
                                    "tsqr::gemm_nn_fused<true>",
                                    "tsqr::tc_tn_tma_kernel<256>",
                                    "tsqr::tc_nn_tma_kernel<128>"])
def test_headline_kernels_do_not_spill(spills, kernel):
    assert kernel not in spills

