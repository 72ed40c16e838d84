"""The drop-in headers include/TallShinnyQR.h and include/block_QR.h keep the
reference's template signatures (TallShinnyQR.h:86-87, block_QR.h:72-73): a
caller written against the reference compiles and links unchanged."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tsqr_gb300", "_build")

CALLER = r"""
#include <cuda_runtime.h>
#include <cstdio>
#include <vector>
#include <random>
#include <algorithm>
#include "block_QR.h"
int main() {
    const int m = 4096, n = 64, ldwork = 2 * 108 * 128;
    std::vector<float> A(m * n), R(n * n);
    std::default_random_engine eng(0U);
    std::uniform_real_distribution<float> dis(-1.0f, 1.0f);
    std::generate(A.begin(), A.end(), [&] { return dis(eng); });
    float *dA, *dR, *dW;
    cudaMalloc(&dA, sizeof(float) * m * n); cudaMalloc(&dR, sizeof(float) * n * n);
    cudaMalloc(&dW, sizeof(float) * ldwork * n);
    cudaMemcpy(dA, A.data(), sizeof(float) * m * n, cudaMemcpyHostToDevice);
    tsqr<float>(m, 32, dA, m, dR, n, dW, ldwork);      // reference signature
    qr<float>(m, n, dA, m, dR, n, dW, ldwork);         // reference signature
    cudaDeviceSynchronize();
    cudaMemcpy(R.data(), dR, sizeof(float) * n * n, cudaMemcpyDeviceToHost);
    double s = 0; for (int i = 0; i < n; ++i) s += R[i + i * n] * R[i + i * n];
    std::printf("%s %f\n", cudaGetErrorString(cudaGetLastError()), s);
    return 0;
}
"""


def build_caller(tmp_path):
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                    str(src), "-o", str(exe), "-L", BUILD, "-ltsqr_gb300", "-Wl,-rpath," + BUILD,
                    "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"], check=True)
    return exe


def test_reference_style_caller_compiles_and_links(tg, tmp_path):
    assert build_caller(tmp_path).exists()


@pytest.mark.gpu
def test_reference_style_caller_runs(cuda, tg, tmp_path):
    exe = build_caller(tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("no error"), out.stdout + out.stderr
    # sum of squared diag(R) of a QR of A = ||A||_F^2 for the second call's
    # R on Q-input: columns 0..31 are orthonormal after the first call
    assert float(out.stdout.split()[-1]) > 0
