"""The reference's output cadence (source/main.cpp:381-474), restated in
tests/cli_golden.py, against the frames and log lines its own executable
wrote for the fixtures (tests/golden/cli_*.npz)."""
import pytest

from cli_golden import NAMES, cadence, load


@pytest.mark.parametrize("name", NAMES)
def test_restated_cadence_matches_reference_executable(name):
    dim, files, inputs, log = load(name)
    # the fixture inputs: 10 steps of Dt, a .prof frame every 3 steps, a .vtk frame every 4
    txt = inputs["case.data"].decode().split()
    kv = {txt[i]: txt[i + 1] for i in range(len(txt) - 1) if txt[i] in ("Dt", "OutputInterval", "VtkOutputInterval", "EndTime")}
    names, lines = cadence(0.0, float(kv["Dt"]), float(kv["EndTime"]), float(kv["OutputInterval"]),
                           float(kv["VtkOutputInterval"]))
    assert names == sorted(files)
    assert lines == log
