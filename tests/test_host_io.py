"""Parser, model and writer parity with the reference's unit tests (CPU).

Ports tests/io_test.cpp, tests/qubo_helpers_test.cpp and the example files of
benchmarks/exhaustive_search/examples through the product's C ABI.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.qubo_text import dense_from_text


def test_nodes_is_max_index_plus_one(native, golden_io):
    # io_test.cpp:41-48: header says 100 nodes, file uses 0..2 -> 3.
    m = native.Model.parse(golden_io["parse_ok"]["text"])
    assert m.nodes == golden_io["parse_ok"]["nodes"]


def test_linear_and_quadratic_values(native, golden_io):
    # io_test.cpp:50-68.
    g = golden_io["parse_ok"]
    m = native.Model.parse(g["text"])
    for i, v in g["variables"].items():
        assert m.get_variable(int(i)) == v
    for i, j, v in g["connections"]:
        assert m.get_connection(i, j) == v
    assert m.get_connection(1, 0) == 0.0  # lower-triangle key is absent
    assert m.get_variable(1) == 0.0


def test_lower_triangle_throws(native, golden_io):
    # io_test.cpp:70-83.
    with pytest.raises(native.ParseError) as e:
        native.Model.parse(golden_io["lower_triangle"])
    assert "lower triangle" in e.value.message


@pytest.mark.parametrize("idx", range(5))
def test_grammar_violations_throw(native, golden_io, idx):
    # io_test.cpp:21-37,85-92.
    with pytest.raises(native.ParseError):
        native.Model.parse(golden_io["grammar_errors"][idx])


def test_quadratic_count_mismatch_throws(native, golden_io):
    # io_test.cpp:94-106.
    with pytest.raises(native.ParseError) as e:
        native.Model.parse(golden_io["quadratic_count"])
    assert "quadratic" in e.value.message


def test_saved_solution_bytes(native, golden_io):
    # io_test.cpp:108-118.
    g = golden_io["csv"]
    assert native.solution_csv(g["state"], g["energy"]) == g["expected"]


@pytest.mark.parametrize("energy,text", [(-1.2, "-1.2"), (1234567.0, "1.23457e+06"), (0.0, "0"),
                                         (-235.8666540000, "-235.867")])
def test_solution_energy_precision(native, energy, text):
    assert native.solution_csv([1, 0], energy).splitlines()[1] == "1,0," + text


def test_flatten_matches_oracle_on_examples(native, orc, golden_exhaustive):
    for name, text in golden_exhaustive["examples"].items():
        if name == "dwave_doc.qubo":
            continue
        m = native.Model.parse(text)
        assert np.array_equal(m.flatten(), dense_from_text(text)), name


def test_dwave_doc_example_is_rejected(native, golden_exhaustive):
    # "p  qubo" has two spaces; the grammar's literal "p qubo" has one
    # (include/model/qubo.hpp:403), which is consistent with the 0.010 s
    # "runtime" in benchmarks/exhaustive_search/perfomance.md:15.
    with pytest.raises(native.ParseError):
        native.Model.parse(golden_exhaustive["examples"]["dwave_doc.qubo"])


@pytest.mark.parametrize("text,ok", [
    ("p qubo 0 2 1 1\n0 0 1\n0 1 2", True),                 # no final newline
    ("p qubo 0 2 1 1\r\n0 0 1\r\n0 1 2\r\n", True),         # CRLF
    ("c a\nc b\np qubo 0 2 1 1\nc mid\n0 0 1\n0 1 2\n", True),
    ("p qubo 0 2 1 1\n0   1 2\n0 0 1\n", True),             # extra blanks before an index
    ("p qubo 0 2 1 1\n0 0 1\n\n0 1 2\n", False),            # empty line
    ("p  qubo 0 2 1 1\n0 0 1\n0 1 2\n", False),             # two spaces in the literal
    ("p qubo 0 2 1 1\n0\t1 2\n0 0 1\n", False),             # tab right after an index
    ("p qubo 0 2 1 1\n0 0 1\n0 1 2 3\n", False),            # extra field
    ("p qubo 0 2 1 1\n0 0 1e-1\n0 1 -.5\n", True),          # exponent, leading dot
    ("p qubo 0 1 1 0\n", False),                            # empty input
    ("0 0 1\n", False),                                     # no header
    ("p qubo 0 1 2 0\n0 0 1\n1 1 2\n", False),              # more linear terms than nodes
])
def test_grammar_edge_cases(native, text, ok):
    if ok:
        native.Model.parse(text)
    else:
        with pytest.raises(native.ParseError):
            native.Model.parse(text)


def test_first_duplicate_key_wins(native):
    m = native.Model.parse("p qubo 0 2 1 1\n0 0 1\n0 0 7\n0 1 2\n")
    assert m.get_variable(0) == 1.0


def test_load_file(native, tmp_path, golden_exhaustive):
    p = tmp_path / "t.qubo"
    p.write_text(golden_exhaustive["examples"]["test1.qubo"])
    assert native.Model.load(p).nodes == 4
    with pytest.raises(native.OneSolverError):
        native.Model.load(tmp_path / "missing.qubo")


def test_device_selector_strings(native):
    # devices_test.cpp: host/cpu/gpu are the accepted strings; this library has
    # no CPU backend, so host/cpu are refused with UNSUPPORTED.
    for t in ("host", "cpu"):
        with pytest.raises(native.OneSolverError) as e:
            native.select_device(t)
        assert e.value.status == native.UNSUPPORTED
    with pytest.raises(native.OneSolverError) as e:
        native.select_device("fpga")
    assert e.value.status == native.INVALID_ARG
    assert "Unknown device type: fpga" in e.value.message
