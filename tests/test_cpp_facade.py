"""The C++ façade (include/vfps.hpp) and the main.cpp-shaped driver built
on it: it compiles warning-free, reads every key the run-file writer
emits, and fails cleanly (status 1, a message) without a GPU."""
import os
import re
import subprocess
import tempfile

import pytest

from inovesa_gb300 import build as B
from inovesa_gb300 import params as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "inovesa_gb300", "cpp", "vfps_solver.cpp")


def test_driver_builds():
    exe = B.build_driver()
    assert os.access(exe, os.X_OK)


def test_run_file_has_every_key_the_driver_reads():
    src = open(SRC).read()
    keys = set(re.findall(r'get\(p, "([A-Za-z_0-9]+)"\)', src))
    assert "n" in keys and "steps" in keys
    p = P.derive(GridSize=64, StepsPerTs=500, padding=2.0)
    text = P.run_file(p, chain=0, steps=3, csr=True)
    have = {ln.split("=")[0].strip() for ln in text.splitlines()}
    assert keys <= have, keys - have
    assert "slip0" in have


def test_driver_reports_missing_device(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = B.build_driver()
    p = P.derive(GridSize=64, StepsPerTs=500, padding=2.0)
    rf = tmp_path / "run.txt"
    rf.write_text(P.run_file(p, steps=1))
    r = subprocess.run([exe, str(rf), str(tmp_path / "out")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "vfps_solver:" in r.stderr
