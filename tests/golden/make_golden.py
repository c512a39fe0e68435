"""Generate the golden fixtures in tests/golden/ from the reference checkout.

Run once where the reference (quantumz-io/oneSolver) is available:

    python tests/golden/make_golden.py /path/to/oneSolver

It extracts, as data, the reference's own known-answer tests and example
instances, so the test suite can run where the reference is absent:

* exhaustive_golden.json -- the five instances and minimum energies of
  tests/exhaustive_test.cpp:12-142 (the same files ship as
  benchmarks/exhaustive_search/examples/*.qubo), plus the other example files;
* io_golden.json -- the parser and writer cases of tests/io_test.cpp:12-118,
  the flatten layout of tests/qubo_helpers_test.cpp:12-30 and the str() case of
  tests/qubo_test.cpp:42-55;
* chimera_128_001.qubo / chimera_512_001.qubo -- the QUBO-form Chimera droplet
  instances of benchmarks/annealing/chimera_droplets_qbsolv (written by the
  reference's converter, benchmarks/annealing/scripts/convert_qbsolv_to_coo.py,
  from chimera_{128,512}_001_ising.txt = benchmarks/annealing/chimera_droplets),
  chimera_golden.json with the published best SA energies
  (benchmarks/annealing/results/*/001.csv) and the tensor-network ground
  states (results/*/groundstates_TN.txt) converted to QUBO energies with
  x = (s + 1) / 2 and the offset dropped (benchmarks/annealing/plot.py:28-38).
"""
from __future__ import annotations

import ast
import csv
import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def cpp_string_literals(block: str) -> str:
    """Concatenate the adjacent C++ string literals in a source block."""
    parts = re.findall(r'"((?:[^"\\]|\\.)*)"', block)
    return "".join(ast.literal_eval('"' + p + '"') for p in parts)


def exhaustive_cases(ref: Path) -> list[dict]:
    src = (ref / "tests" / "exhaustive_test.cpp").read_text()
    cases = []
    for m in re.finditer(r"std::make_pair<std::string, double>\((.*?),\s*(-?[0-9.]+)\)", src, re.S):
        cases.append({"text": cpp_string_literals(m.group(1)), "energy": float(m.group(2))})
    return cases


def io_cases(ref: Path) -> dict:
    src = (ref / "tests" / "io_test.cpp").read_text()
    good = re.search(r"qubo_file_contents\((.*?)\);", src, re.S).group(1)
    bad_block = re.search(r"grammatically_incorrect_file_contents\[\]\{(.*?)\};", src, re.S).group(1)
    bad = [cpp_string_literals(b) for b in re.findall(r"std::string\((.*?)\)", bad_block, re.S)]
    reversed_case = re.search(
        r"reversed_order\)\s*\{\s*std::string invalid_qubo_file_contents\((.*?)\);", src, re.S).group(1)
    count_case = re.search(
        r"declared_one\)\s*\{\s*std::string invalid_qubo_file_contents\((.*?)\);", src, re.S).group(1)
    csv_expected = cpp_string_literals(re.search(r"expected_output = (.*?);", src, re.S).group(1))
    state = [int(v) for v in re.search(r"char state\[\] = \{(.*?)\}", src).group(1).split(",")]
    energy = float(re.search(r"solution\(state, state \+ \d+, (-?[0-9.]+)\)", src).group(1))

    hsrc = (ref / "tests" / "qubo_helpers_test.cpp").read_text()
    lin = re.search(r"linear_c\{(.*?)\};", hsrc, re.S).group(1)
    lin_pairs = [(int(a), float(b)) for a, b in re.findall(r"\{(\d+),\s*(-?[0-9.]+)\}", lin)]
    quad = re.search(r"quadratic_c\{(.*?)\};", hsrc, re.S).group(1)
    quad_pairs = [(int(a), int(b), float(c))
                  for a, b, c in re.findall(r"std::pair\((\d+),\s*(\d+)\),\s*(-?[0-9.]+)\}", quad)]
    n_nodes = int(re.search(r"set_nodes\((\d+)\)", hsrc).group(1))
    expected = [float(v) for v in re.search(r"expected_result\(\s*\{(.*?)\}\)", hsrc, re.S).group(1).split(",")]

    qsrc = (ref / "tests" / "qubo_test.cpp").read_text()
    str_expected = re.search(r's\.compare\("(.*?)"\)', qsrc).group(1)
    return {
        "parse_ok": {"text": cpp_string_literals(good), "nodes": 3,
                     "variables": {"0": -0.5, "2": -0.7}, "connections": [[0, 1, 2.0], [1, 2, 4.0]]},
        "grammar_errors": bad,
        "lower_triangle": cpp_string_literals(reversed_case),
        "quadratic_count": cpp_string_literals(count_case),
        "csv": {"state": state, "energy": energy, "expected": csv_expected},
        "flatten": {"n": n_nodes, "linear": lin_pairs, "quadratic": quad_pairs, "expected": expected},
        "str": {"linear": [[1, 10]], "quadratic": [[1, 2, 20]], "expected": str_expected},
    }


def example_files(ref: Path) -> dict:
    ex = ref / "benchmarks" / "exhaustive_search" / "examples"
    return {p.name: p.read_text() for p in sorted(ex.glob("*.qubo"))}


def tn_qubo_energy(qubo_text: str, tn_line: str) -> float:
    """QUBO energy of the published +/-1 ground state, x = (s + 1) / 2."""
    spins = [int(v) for v in tn_line.split(":", 1)[1].split()[1:]]
    x = [(s + 1) // 2 for s in spins]
    e = 0.0
    for line in qubo_text.splitlines():
        if not line or line[0] in "cp":
            continue
        i, j, v = line.split()
        i, j = int(i), int(j)
        if x[i] and x[j]:
            e += float(v)
    return e


def chimera(ref: Path) -> dict:
    out = {}
    base = ref / "benchmarks" / "annealing"
    for size in (128, 512):
        text = (base / "chimera_droplets_qbsolv" / f"{size}power" / "001.txt").read_text()
        (HERE / f"chimera_{size}_001.qubo").write_text(text)
        # the Ising original the reference's converter turned into the file above
        ising = (base / "chimera_droplets" / f"{size}power" / "001.txt").read_text()
        (HERE / f"chimera_{size}_001_ising.txt").write_text(ising)
        tn = (base / "results" / str(size) / "groundstates_TN.txt").read_text().splitlines()[0]
        with open(base / "results" / str(size) / "001.csv") as fh:
            best = min(float(row["energy"]) for row in csv.DictReader(fh))
        out[str(size)] = {"file": f"chimera_{size}_001.qubo", "tn_ground_qubo": tn_qubo_energy(text, tn),
                          "published_best_sa": best}
    return out


def main(ref: Path) -> None:
    (HERE / "exhaustive_golden.json").write_text(json.dumps(
        {"cases": exhaustive_cases(ref), "examples": example_files(ref)}, indent=1))
    (HERE / "io_golden.json").write_text(json.dumps(io_cases(ref), indent=1))
    (HERE / "chimera_golden.json").write_text(json.dumps(chimera(ref), indent=1))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the oneSolver reference checkout>")
    main(Path(sys.argv[1]))
