"""CsvWriter's nodal CSV (src/io/csv_writer.cpp:34-57), host only: the header,
one line per node in ascending node-id order for each subcase in the order
given, values in scientific notation with 8 digits after the point, and the
reference's error text for a file that cannot be written."""
import numpy as np
import pytest


def test_write_node_csv_format(vsgb, tmp_path):
    ids = np.array([7, 3, 12, 5], np.int32)
    disp = (np.arange(2 * 4 * 6, dtype=float).reshape(2, 4, 6) - 20.0) * 1.2345678901e-4
    disp[1, 2, 4] = -0.0
    path = tmp_path / "case.node.csv"
    vsgb.write_node_csv(str(path), ids, disp, [1, 4])
    lines = path.read_text().splitlines()
    exp = ["# node_id, subcase_id, T1, T2, T3, R1, R2, R3"]
    for s, sc in enumerate((1, 4)):
        for i in np.argsort(ids, kind="stable"):
            exp.append(f"{ids[i]}, {sc}, " + ", ".join(f"{v:.8e}" for v in disp[s, i]))
    assert lines == exp


def test_write_node_csv_errors(vsgb, tmp_path):
    ids = np.array([1, 2], np.int32)
    with pytest.raises(vsgb.SolverError, match="Cannot write CSV: .*x.node.csv"):
        vsgb.write_node_csv(str(tmp_path / "missing" / "x.node.csv"), ids, np.zeros((2, 6)))
    with pytest.raises(vsgb.SolverError, match="one subcase id"):
        vsgb.write_node_csv(str(tmp_path / "y.csv"), ids, np.zeros((2, 2, 6)), [1])
