"""Generate golden vectors from the reference's OWN CUDA kernels.

Run on a GPU host after build() (needs oracle/_ref/ref_kernels.cubin, which
build() compiles unmodified from the reference checkout):

    python tests/golden/make_golden.py [outdir]

For each case it draws the reference's input (std::default_random_engine(0)
+ uniform_real_distribution(-1, 1), column-major, test_tsqr.cu:24-28), runs
the reference tsqr / qr host schedule (restated in oracle/ref_launch.cpp,
kernels from the cubin), and stores a small fixture:
  R                the full n x n R the reference wrote
  q_rows, q_idx    Q at 512 fixed rows (the first 256 and 256 spread rows)
  q_colsum         FP64 column sums of the full Q
  m, n, kind, dtype
Fixtures are compared with the oracle restatement (CPU, test_golden.py) and
with libtsqr_gb300 (GPU, test_tsqr_gpu.py::test_matches_reference_cuda_golden).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

CASES = [
    ("tsqr", "float32", 128, 32), ("tsqr", "float32", 1024, 32), ("tsqr", "float32", 13824, 32),
    ("tsqr", "float32", 27648, 32), ("tsqr", "float32", 4096, 16), ("tsqr", "float32", 2048, 8),
    ("tsqr", "float32", 100000, 32),
    ("tsqr", "float64", 1024, 32), ("tsqr", "float64", 27648, 32),
    ("qr", "float32", 27648, 128), ("qr", "float64", 27648, 128), ("qr", "float32", 4096, 64),
]


def sample_rows(m):
    idx = list(range(min(m, 256)))
    if m > 256:
        idx += list(np.linspace(256, m - 1, 256).astype(np.int64))
    return np.array(sorted(set(idx)), dtype=np.int64)


def main(outdir):
    import torch
    from oracle import oracle as orc
    os.makedirs(outdir, exist_ok=True)
    for kind, dt, m, n in CASES:
        dtype = np.float32 if dt == "float32" else np.float64
        tdt = torch.float32 if dt == "float32" else torch.float64
        A = orc.fill_uniform(m, n, dtype)
        dA = torch.from_numpy(np.ascontiguousarray(A.T)).to("cuda")  # (n, m) rows = columns
        dR = torch.zeros((n, n), dtype=tdt, device="cuda")
        work = torch.zeros(orc.REF_LDWORK * n, dtype=tdt, device="cuda")
        torch.cuda.synchronize()
        rc = orc.ref_cuda_call(kind, dA, dR, work)
        torch.cuda.synchronize()
        if rc != 0:
            raise SystemExit("reference launcher refused %s %s %dx%d: rc=%d" % (kind, dt, m, n, rc))
        Q = dA.cpu().numpy().T
        R = dR.cpu().numpy().T
        idx = sample_rows(m)
        name = os.path.join(outdir, "ref_%s_%s_%dx%d.npz" % (kind, dt, m, n))
        np.savez_compressed(name, R=np.asfortranarray(R), q_rows=Q[idx], q_idx=idx,
                            q_colsum=Q.astype(np.float64).sum(axis=0), m=m, n=n, kind=kind, dtype=dt)
        met = orc.metrics(A, np.asfortranarray(Q), np.asfortranarray(R))
        print(name, met)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
