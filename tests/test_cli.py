"""The test_tsqr / test_qr command lines (drop-ins for the reference's
test_tsqr.cu / test_qr.cu: `m n dtype`, the same printed lines)."""
import json
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tsqr_gb300", "_build")


def test_cli_binaries_built(tg):
    for name in ("test_tsqr", "test_qr"):
        assert os.access(os.path.join(BUILD, name), os.X_OK)


@pytest.mark.gpu
@pytest.mark.parametrize("name,args,n", [("test_tsqr", ["27648", "32", "1"], 32),
                                          ("test_tsqr", ["27648", "32", "2"], 32),
                                          ("test_tsqr", [], 32),
                                          ("test_qr", ["27648", "128", "2"], 128),
                                          ("test_qr", ["27648", "128", "1"], 128)])
def test_cli_output_lines(cuda, tg, name, args, n):
    out = subprocess.run([os.path.join(BUILD, name)] + args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.strip().splitlines()
    m = re.match(r"\|A-QR\|/\|A\| = ([0-9.eE+-]+), \|I-Q\^TQ\| / n = ([0-9.eE+-]+)", lines[0])
    assert m, lines
    back2, orth2 = float(m.group(1)), float(m.group(2))
    single = "1" in args[2:3]
    u = 2.0 ** -24 if single else 2.0 ** -53
    assert back2 <= 10 * n * u and orth2 <= 10 * u * n
    kind = "qr" if name == "test_qr" else "tsqr"
    assert re.match(r"%s Latency: [0-9.]+ ms" % kind, lines[1]), lines
    js = json.loads(lines[2])
    assert js["cli"] == kind and js["tflops"] > 0
