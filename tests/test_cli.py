"""The one-solver-anneal / one-solver-exhaustive command-line tools.

Flags, messages and exit codes follow the reference's app/one-solver-anneal.cpp
(:55-72 options, :83-115 validation, :171-176 errors) and
app/one-solver-exhaustive.cpp; the argument checks run without a GPU, the
solver runs on one.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from onesolver_gb300 import build as nbuild

from qubo_text import dense_from_text, random_int_qubo

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def apps():
    exes = {p.name: p for p in nbuild.build_apps()}
    return exes["one-solver-anneal"], exes["one-solver-exhaustive"]


def run(exe, *args):
    p = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=300)
    return p.returncode, p.stdout, p.stderr


def qubo_text(f: np.ndarray) -> str:
    n = f.shape[0]
    diag = [(i, f[i, i]) for i in range(n) if f[i, i] != 0]
    quad = [(i, j, f[i, j]) for i in range(n) for j in range(i + 1, n) if f[i, j] != 0]
    lines = [f"p qubo 0 {n} {len(diag)} {len(quad)}"]
    lines += [f"{i} {i} {v:.17g}" for i, v in diag] + [f"{i} {j} {v:.17g}" for i, j, v in quad]
    return "\n".join(lines) + "\n"


def read_csv(path: Path):
    head, row = path.read_text().splitlines()[:2]
    cells = row.split(",")
    return [int(c) for c in cells[:-1]], float(cells[-1]), head


@pytest.fixture
def small_input(tmp_path):
    f = random_int_qubo(10, 4)
    # keep every diagonal entry non-zero so that the node count is n
    np.fill_diagonal(f, np.where(np.diag(f) == 0, 1.0, np.diag(f)))
    path = tmp_path / "in.qubo"
    path.write_text(qubo_text(f))
    return f, path


def test_help_lists_the_reference_options(apps):
    anneal, exh = apps
    rc, out, _ = run(anneal, "--help")
    assert rc == 0
    for opt in ("--input", "--output", "--num-iter", "--num-tries", "--schedule-type", "--beta-min", "--beta-max",
                "--device-type", "--sweeps-per-beta"):
        assert opt in out
    rc, out, _ = run(exh, "--help")
    assert rc == 0 and "--input" in out and "--device-type" in out


@pytest.mark.parametrize("which", [0, 1])
def test_missing_files_are_reported(apps, which, tmp_path):
    exe = apps[which]
    rc, _, err = run(exe)
    assert rc == 255 and "No input file provided." in err
    rc, _, err = run(exe, "--input", tmp_path / "x.qubo")
    assert rc == 255 and "No output file provided." in err
    rc, _, err = run(exe, "--input", tmp_path / "missing.qubo", "--output", tmp_path / "o.csv")
    assert rc == 255 and "can not open input file" in err


@pytest.mark.parametrize("which", [0, 1])
def test_device_types(apps, which, small_input, tmp_path):
    exe = apps[which]
    _, path = small_input
    rc, _, err = run(exe, "--input", path, "--output", tmp_path / "o.csv", "--device-type", "fpga")
    assert rc == 255 and "Unknown device type: fpga" in err
    # host and cpu are valid names without a backend in this library
    for dev in ("host", "cpu"):
        rc, _, err = run(exe, "--input", path, "--output", tmp_path / "o.csv", "--device-type", dev)
        assert rc == 1 and "No devices of given type could be initialized." in err


@pytest.mark.parametrize("args,msg", [
    (("--schedule-type", "cosine"), "Unknown beta schedule: cosine"),
    (("--beta-min", "2", "--beta-max", "1"), "initial beta is not lesser than final beta"),
    (("--beta-min", "-1"), "both ends of beta range need to be positive"),
    (("--site-order", "spiral"), "Unknown site order: spiral"),
    (("--acceptance", "glauber"), "Unknown acceptance rule: glauber"),
])
def test_anneal_argument_checks(apps, small_input, tmp_path, args, msg):
    _, path = small_input
    rc, _, err = run(apps[0], "--input", path, "--output", tmp_path / "o.csv", *args)
    assert rc == 255 and msg in err


def test_malformed_input_is_an_error(apps, tmp_path):
    path = tmp_path / "bad.qubo"
    path.write_text("p qubo 0 100 3 492\n0 0 -0.5\nunexpected string\n0 1 2.0\n")
    for exe in apps:
        rc, _, err = run(exe, "--input", path, "--output", tmp_path / "o.csv")
        assert rc == 1 and err.startswith("error: ")


@pytest.mark.gpu
def test_exhaustive_cli_matches_oracle(apps, small_input, tmp_path):
    f, path = small_input
    out, allp = tmp_path / "o.csv", tmp_path / "all.csv"
    rc, stdout, err = run(apps[1], "--input", path, "--output", out, "--all-minimisers", allp)
    assert rc == 0, err
    assert "Using device:" in stdout
    bits, energy, head = read_csv(out)
    n = f.shape[0]
    assert head == ",".join(map(str, range(n))) + ",energy"
    e, count, states = oracle.exhaustive_all(f, 0, 1 << n)
    assert out.read_text().splitlines()[1].split(",")[-1] == f"{e:g}"
    assert sum(b << i for i, b in enumerate(bits)) == int(states[0])
    rows = allp.read_text().splitlines()[1:]
    assert len(rows) == count


@pytest.mark.gpu
def test_anneal_cli_on_the_chimera_fixture(apps, tmp_path):
    src = ROOT / "tests" / "golden" / "chimera_128_001.qubo"
    f = dense_from_text(src.read_text())
    out = tmp_path / "o.csv"
    rc, stdout, err = run(apps[0], "--input", src, "--output", out, "--num-iter", "200", "--num-tries", "64",
                          "--beta-min", "0.1", "--beta-max", "3", "--site-order", "sequential",
                          "--acceptance", "physical", "--resync-every", "50")
    assert rc == 0, err
    assert "Number of tries: 64" in stdout
    bits, energy, _ = read_csv(out)
    assert len(bits) == f.shape[0]
    # Solution::save writes the energy with the stream's default precision
    # (six significant digits, solution.hpp:58-67).
    e = oracle.energy(f, np.array(bits, dtype=np.uint8))
    assert out.read_text().splitlines()[1].split(",")[-1] == f"{e:g}"


# ---------------------------------------------------------------------------
# one-solver-temper (parallel tempering; no reference counterpart)
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def temper():
    return {p.name: p for p in nbuild.build_apps()}["one-solver-temper"]


def test_temper_help_and_checks(temper, small_input, tmp_path):
    rc, out, _ = run(temper, "--help")
    assert rc == 0
    for opt in ("--input", "--output", "--method", "--population", "--num-temps", "--num-chains", "--num-rounds",
                "--sweeps-per-round",
                "--beta-min", "--beta-max", "--device-type", "--seed", "--resync-every"):
        assert opt in out
    rc, _, err = run(temper)
    assert rc == 255 and "No input file provided." in err
    _, path = small_input
    for args, msg in [(("--beta-min", "2", "--beta-max", "1"), "beta-min is greater than beta-max"),
                      (("--beta-min", "0"), "both ends of beta range need to be positive"),
                      (("--num-temps", "0"), "num-temps must be positive"),
                      (("--method", "qmc"), "Unknown method: qmc"),
                      (("--device-type", "fpga"), "Unknown device type: fpga")]:
        rc, _, err = run(temper, "--input", path, "--output", tmp_path / "o.csv", *args)
        assert rc == 255 and msg in err, (args, err)
    rc, _, err = run(temper, "--input", path, "--output", tmp_path / "o.csv", "--device-type", "host")
    assert rc == 1 and "No devices of given type could be initialized." in err


@pytest.mark.gpu
def test_temper_cli_reaches_the_droplet_ground_state(temper, tmp_path, golden_chimera):
    src = ROOT / "tests" / "golden" / "chimera_128_001.qubo"
    f = dense_from_text(src.read_text())
    out = tmp_path / "o.csv"
    rc, stdout, err = run(temper, "--input", src, "--output", out, "--num-chains", "64", "--num-rounds", "800")
    assert rc == 0, err
    assert "Using device:" in stdout
    bits, energy, _ = read_csv(out)
    e = oracle.energy(f, np.array(bits, dtype=np.uint8))
    assert abs(e - golden_chimera["128"]["tn_ground_qubo"]) < 1e-6
    assert out.read_text().splitlines()[1].split(",")[-1] == f"{e:g}"


@pytest.mark.gpu
def test_temper_cli_population_annealing(temper, tmp_path, golden_chimera):
    src = ROOT / "tests" / "golden" / "chimera_128_001.qubo"
    f = dense_from_text(src.read_text())
    out = tmp_path / "o.csv"
    rc, stdout, err = run(temper, "--input", src, "--output", out, "--method", "pa", "--num-temps", "300",
                          "--population", "8192")
    assert rc == 0, err
    assert "Population: 8192" in stdout
    bits, energy, _ = read_csv(out)
    e = oracle.energy(f, np.array(bits, dtype=np.uint8))
    assert abs(e - golden_chimera["128"]["tn_ground_qubo"]) < 1e-6
