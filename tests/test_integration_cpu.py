"""The cellBP drop-in (wholecellfe_gb300/shim) compiles against the reference's headers and
links with the reference's own declarations of the mechanics functions and libwcfe.so
(oracle/check_integration.sh).  Runs where the reference sources are available (the
container that builds oracle/_ref); skipped elsewhere.  No GPU."""
import os
import subprocess

import pytest

from oracle import oracle_py as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integration_shim_compiles_and_links():
    if not O.ref_available("kMD"):
        pytest.skip("reference not built here (oracle/build_ref.sh)")
    r = subprocess.run(["sh", os.path.join(ROOT, "oracle", "check_integration.sh")], capture_output=True, text=True,
                       timeout=600)
    if r.returncode == 77:
        pytest.skip(r.stderr.strip())
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compiles and links" in r.stdout
