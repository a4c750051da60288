"""The generated per-point algebra (product code) compiled for the host and
checked against the oracle's point function on random inputs: catches a
generator error before any GPU run."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dendro-5.01_gb300", "csrc")


def test_ccz4_algebra_matches_oracle_point(oracle, tmp_path):
    import oracle_py
    exe = tmp_path / "ccz4_algebra_check"
    src = os.path.join(ROOT, "tests", "host", "ccz4_algebra_check.cpp")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, "-o", str(exe), src,
                        oracle_py.ORACLE_SO, f"-Wl,-rpath,{os.path.dirname(oracle_py.ORACLE_SO)}",
                        "-lm"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr[-2000:])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    sys.stdout.write(out.stdout)
    assert out.returncode == 0, out.stdout


def test_bssn_algebra_matches_oracle_point(oracle, tmp_path):
    """Both BSSN algebras (centred advection; the upwinded sums of the 4th-order
    binding) against orc_bssn_point."""
    import oracle_py
    exe = tmp_path / "bssn_algebra_check"
    src = os.path.join(ROOT, "tests", "host", "bssn_algebra_check.cpp")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, "-o", str(exe), src,
                        oracle_py.ORACLE_SO, f"-Wl,-rpath,{os.path.dirname(oracle_py.ORACLE_SO)}",
                        "-lm"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr[-2000:])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    sys.stdout.write(out.stdout)
    assert out.returncode == 0, out.stdout
