"""The integer hi/lo split of the mixed path gives the same bits as the FP64 subtraction route
(tests/native/split_hl_check.cpp, compiled with the host compiler). CPU only."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_split_matches_fp64_route():
    d = tempfile.mkdtemp(prefix="split_")
    exe = os.path.join(d, "split_hl_check")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "split_hl_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    assert "bad 0" in out, out
