"""Ising -> QUBO conversion (os_ising_to_qubo_text, one-solver-ising2qubo)
against the reference's own converted files.

The reference converted its Chimera droplet instances with
benchmarks/annealing/scripts/convert_qbsolv_to_coo.py (dimod); both the Ising
originals and the QUBO files it wrote are committed fixtures, so the
conversion is pinned on the reference's output, byte for byte. A brute-force check ties the
offset: E_ising(s) = E_qubo(x) + offset with s = 2x - 1.
"""
from __future__ import annotations

import itertools
import subprocess
from pathlib import Path

import numpy as np
import pytest

import onesolver_gb300 as osg
from onesolver_gb300 import build as nbuild

GOLDEN = Path(__file__).resolve().parent / "golden"


def entries(text: str):
    head, out = None, {}
    for line in text.splitlines():
        s = line.strip()
        if not s or s[0] in "#c":
            continue
        if s.startswith("p"):
            head = s.split()
            continue
        i, j, v = s.split()
        out[(int(i), int(j))] = float(v)
    return head, out


@pytest.mark.parametrize("size", [128, 512])
def test_matches_the_reference_converter(size):
    """Byte for byte: the same header, entries, order and number formatting
    as the file the reference's dimod-based converter wrote."""
    ising = (GOLDEN / f"chimera_{size}_001_ising.txt").read_text()
    ref_text = (GOLDEN / f"chimera_{size}_001.qubo").read_text()
    text, offset = osg.ising_to_qubo_text(ising)
    assert text == ref_text
    head, got = entries(text)
    assert int(head[3]) == size and int(head[5]) == sum(i != j for i, j in got)


def test_energy_identity_and_offset():
    rng = np.random.default_rng(1)
    n = 9
    lines = ["# random Ising model"]
    h = rng.normal(size=n)
    J = {}
    for i in range(n):
        lines.append(f"{i + 1} {i + 1} {float(h[i])!r}")
    for i, j in itertools.combinations(range(n), 2):
        if rng.random() < 0.6:
            J[(i, j)] = float(rng.normal())
            lines.append(f"{j + 1} {i + 1} {J[(i, j)]!r}")  # either order
    text, offset = osg.ising_to_qubo_text("\n".join(lines) + "\n")
    _, q = entries(text)
    for bits in itertools.product([0, 1], repeat=n):
        x = np.array(bits, dtype=float)
        s = 2 * x - 1
        e_ising = float(h @ s) + sum(v * s[i] * s[j] for (i, j), v in J.items())
        e_qubo = sum(v * x[i] * x[j] for (i, j), v in q.items())
        assert e_ising == pytest.approx(e_qubo + offset, abs=1e-9)


@pytest.mark.parametrize("bad", ["1 2\n", "0 1 1.0\n", "1 1 nan\n", "1 2 3 4\n", "# only a comment\n"])
def test_malformed_input_is_rejected(bad):
    with pytest.raises(osg.OneSolverError):
        osg.ising_to_qubo_text(bad)


def test_cli(tmp_path):
    exe = {p.name: p for p in nbuild.build_apps()}["one-solver-ising2qubo"]
    out = tmp_path / "out.qubo"
    p = subprocess.run([str(exe), "--input", str(GOLDEN / "chimera_128_001_ising.txt"), "--output", str(out)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    text, offset = osg.ising_to_qubo_text((GOLDEN / "chimera_128_001_ising.txt").read_text())
    assert out.read_text() == text
    assert float(p.stdout.split()[-1]) == pytest.approx(offset, rel=1e-15)
    p = subprocess.run([str(exe), "--output", str(out)], capture_output=True, text=True, timeout=120)
    assert p.returncode == 255 and "No input file provided." in p.stderr
