"""Host logic of the per-device launch caches in tsqr_gb300/csrc/internal.h:
PerDeviceOnce runs its setup once per device, also under concurrent
callers, and device_sm_count() falls back to a usable count when no
device answers.  Compiled with g++ against the CUDA runtime; the CPU test
runs it where cudaGetDevice fails (no GPU), the GPU test where it succeeds.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cstdio>
#include <thread>
#include <vector>
#include "internal.h"
int main() {
    tsqr::PerDeviceOnce once;
    std::atomic<int> runs{0};
    std::vector<std::thread> th;
    for (int t = 0; t < 8; ++t)
        th.emplace_back([&] { for (int i = 0; i < 1000; ++i) once.run([&] { runs.fetch_add(1); }); });
    for (auto& x : th) x.join();
    const int sms = tsqr::device_sm_count();
    const int again = tsqr::device_sm_count();
    std::printf("%d %d %d %d\n", runs.load(), sms, again, tsqr::current_device());
    return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    d = tmp_path_factory.mktemp("caches")
    src = d / "caches.cpp"
    src.write_text(PROG)
    exe = d / "caches"
    subprocess.run(["g++", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "tsqr_gb300", "csrc"),
                    "-I", "/usr/local/cuda/include", str(src), "-o", str(exe), "-L/usr/local/cuda/lib64",
                    "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"], check=True)
    return exe


def _run(exe):
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return [int(x) for x in out.stdout.split()]


def test_once_per_device_without_gpu(prog):
    import torch
    if torch.cuda.is_available():
        pytest.skip("runs where no device answers")
    runs, sms, again, dev = _run(prog)
    assert runs == 1 and dev == 0
    assert sms == again == 148  # the fallback count


@pytest.mark.gpu
def test_once_per_device_on_gpu(prog, cuda):
    import torch
    runs, sms, again, dev = _run(prog)
    assert runs == 1 and dev == 0
    assert sms == again == torch.cuda.get_device_properties(0).multi_processor_count
