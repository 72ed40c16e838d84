"""Time the reference's own CUDA kernels on a GPU host (test infrastructure).

    python oracle/ref_bench.py [--reps 5]

Runs the reference tsqr / qr host schedules (restated in
oracle/ref_launch.cpp) over the reference's kernels compiled unmodified into
oracle/_ref/ref_kernels.cubin, on the reference's own input stream, and
prints one JSON line per case with the mean device time (CUDA events around
the call, A re-uploaded before each call outside the timed region, as the
reference drivers do: test_tsqr.cu:74-87) and TFLOP/s by F = 4mn^2 - 4/3 n^3.
Only the sizes the reference supports and that ran safely are timed (n = 32
for tsqr; see ref_launch.cpp for the checks made before every launch).
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

CASES = [("tsqr", "float32", 27648, 32), ("tsqr", "float64", 27648, 32), ("tsqr", "float32", 4194304, 32),
         ("qr", "float32", 27648, 128), ("qr", "float64", 27648, 128)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    import numpy as np
    import torch
    from oracle import oracle as orc
    if not orc.ref_cuda_available():
        print(json.dumps({"unavailable": "oracle/_ref/ref_kernels.cubin not built"}))
        return 0
    for kind, dt, m, n in CASES:
        tdt = torch.float32 if dt == "float32" else torch.float64
        A = orc.fill_uniform(m, n, np.float32 if dt == "float32" else np.float64)
        A0 = torch.from_numpy(np.ascontiguousarray(A.T)).to("cuda")
        dA = A0.clone()
        dR = torch.zeros((n, n), dtype=tdt, device="cuda")
        work = torch.zeros(orc.REF_LDWORK * n, dtype=tdt, device="cuda")
        ts = []
        for k in range(args.reps + 2):
            dA.copy_(A0)
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            rc = orc.ref_cuda_call(kind, dA, dR, work)
            e.record()
            torch.cuda.synchronize()
            if rc != 0:
                raise SystemExit("launcher refused %s %dx%d rc=%d" % (kind, m, n, rc))
            if k >= 2:
                ts.append(s.elapsed_time(e))
        ms = sum(ts) / len(ts)
        F = 4.0 * m * n * n - 4.0 / 3.0 * n ** 3
        print(json.dumps({"impl": "reference CUDA (unmodified kernels, sm_103a)", "kind": kind, "dtype": dt,
                          "m": m, "n": n, "ms": ms, "tflops": F / (ms * 1e-3) / 1e12}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
