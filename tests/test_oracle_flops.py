"""The element-assembly work unit: the oracle's membrane element (A3, evalElementRe
UL:710-928 for the cell, UL:989-1176 for the substrate), compiled with a counting scalar
in place of double (oracle/flop_count.cpp), performs exactly this many floating-point
operations (add, subtract, multiply, divide, sqrt; exp and acos do not occur)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "..", "oracle", "flop_count.cpp")

ELEMENT_CELL = dict(add=880, mul=1414, div=62, sqrt=4, exp=0, acos=0, flops=2360)
ELEMENT_SUBSTRATE = dict(add=851, mul=1372, div=59, sqrt=3, exp=0, acos=0, flops=2285)


def test_element_flop_count(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "flop_count")
    subprocess.run([gxx, "-std=c++17", "-O1", "-o", exe, SRC], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    counts = {}
    for line in out:
        if not line.strip():
            continue
        name, *kv = line.split()
        counts[name] = {k: int(v) for k, v in (t.split("=") for t in kv)}
    for name, want in (("element_cell", ELEMENT_CELL), ("element_substrate", ELEMENT_SUBSTRATE)):
        got = counts[name]
        assert {k: got[k] for k in want} == want, (name, got)
