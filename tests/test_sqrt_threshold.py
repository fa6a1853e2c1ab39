"""The bond builder and the contact test decide sqrt(s) <= delta as s <= sqrt_le_max(delta)
(perigrain_gb300/csrc/pg_sqrt_threshold.h): both forms agree on every s around delta^2, random s,
special values and deltas of every magnitude (tests/native/sqrt_threshold_check.cpp, compiled with
the host compiler). CPU only."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "perigrain_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_threshold_matches_sqrt_rule():
    d = tempfile.mkdtemp(prefix="sqrtthr_")
    exe = os.path.join(d, "sqrt_threshold_check")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "native", "sqrt_threshold_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "100000"], capture_output=True, text=True, timeout=300).stdout
    assert out.strip().endswith("bad 0"), out
