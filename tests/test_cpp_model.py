"""Compile and run the C++ port of the reference's model unit tests (CPU)."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_cpp_model_unit_tests(tmp_path):
    exe = tmp_path / "model_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "model_test.cpp"), "-o", str(exe)], check=True)
    proc = subprocess.run([str(exe)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert proc.stdout.strip() == "ok"


def test_cpp_tempering_host_pieces(tmp_path):
    exe = tmp_path / "tempering_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "tempering_test.cpp"), "-o", str(exe)], check=True)
    proc = subprocess.run([str(exe)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert proc.stdout.strip() == "ok"
