"""The reference-side bindings of INTEGRATION.md compile against the
reference's own headers (oracle/check_integration.py: g++ -fsyntax-only on
the stand-in Eigen / Boost headers, -Werror=missing-declarations so that a
binding whose signature differs from the reference's declaration fails)."""
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_integration_bindings_compile():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "check_integration.py")],
                       capture_output=True, text=True)
    if r.returncode == 2:
        pytest.skip(r.stdout.strip())  # no reference checkout on this machine
    assert r.returncode == 0, r.stdout + r.stderr
