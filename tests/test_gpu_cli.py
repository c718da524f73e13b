"""The command-line drop-in (mphimplicit_gb300/_lib/mph_gb300, the
reference's argv) against the reference executable on the same input files:
the same frame files (output.vtk, .prof every OutputInterval, .vtk every
VtkOutputInterval, numbered by step), the same output lines in the log, and
frames with the reference writer's layout (writeProfFile main.cpp:696-720,
writeVtkFile main.cpp:722-883): header, section order and labels, integer
data (types, cells, neighbour counts) identical; floating-point data
(printed to 7 digits from float casts) within 1e-5 of each section's largest
magnitude after 10 steps.  The fixtures (tests/golden/cli_*.npz) come from
the reference's own executables."""
import os
import subprocess

import pytest

from cli_golden import NAMES, compare_frame, load
from mphimplicit_gb300 import build

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", NAMES)
def test_cli_frames_match_reference_executable(engine_lib, name, tmp_path):
    dim, files, inputs, log = load(name)
    for fn, data in inputs.items():
        (tmp_path / fn).write_bytes(data)
    r = subprocess.run([build.CLI_PATH, f"-{dim}", "case.data", "case.grid", "prof%03d.prof", "vtk%03d.vtk", "case.log", "1"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = sorted(f for f in os.listdir(tmp_path) if f.endswith(".prof") or f.endswith(".vtk"))
    assert got == sorted(files)
    lines = [ln for ln in (tmp_path / "case.log").read_text().splitlines() if ln.startswith("@ ")]
    assert lines == log
    worst = {}
    for fn, ref in files.items():
        dev = compare_frame((tmp_path / fn).read_text(), ref, 1e-5)
        for k, v in dev.items():
            worst[k] = max(worst.get(k, 0.0), v)
    print(f"{name}: largest relative deviation per section {worst}")
