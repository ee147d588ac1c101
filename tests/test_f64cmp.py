"""The float64 comparisons by integer operations of the antialiased line
kernels (csrc/f64cmp.cuh), checked on the host: each helper against the IEEE
operation it replaces over special values (signed zeros, subnormals, the
largest finite, infinities, NaNs of both signs and several payloads) and
random ones, and the uint32 -> float64 conversion against the C conversion.
The scanline span ends decided by the float32 intercept (csrc/aa_scan.cuh)
against the float64 intercept's ceil / floor, and the float32 pixel
classification of the queued line kernel against the float64 tests."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "datashader_gb300", "csrc")


def test_f64cmp_helpers_match_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "f64cmp_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}",
                    os.path.join(HERE, "f64cmp_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")


def _run_check(tmp_path, src):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / src.replace(".cpp", ""))
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}",
                    os.path.join(HERE, src), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
    return r.stdout


def test_aa_scan_span_matches_float64(tmp_path):
    out = _run_check(tmp_path, "aa_scan_check.cpp")
    share = float(out.split()[3])
    assert share > 0.5, out          # most scanline ends are decided in float32
    assert float(out.split()[-4]) > 0.9, out    # and most pixels are classified in float32
