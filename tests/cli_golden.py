"""Helpers of the command-line / frame parity tests: the fixtures written by
tests/golden/make_golden.py from the reference executables, the reference's
output cadence restated, and a tolerant comparison of .vtk / .prof frames."""
from __future__ import annotations

import json
import os
from typing import Dict, List, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("dam2d", "cube3d")


def load(name: str):
    z = np.load(os.path.join(HERE, "golden", f"cli_{name}.npz"))
    files = {k[5:]: bytes(z[k]).decode() for k in z.files if k.startswith("file:")}
    inputs = {k[6:]: bytes(z[k]) for k in z.files if k.startswith("input:")}
    return int(z["dim"]), files, inputs, json.loads(str(z["log"]))


def cadence(time0: float, dt: float, end: float, out_iv: float, vtk_iv: float) -> Tuple[List[str], List[str]]:
    """Frame names and output log lines of the reference's time loop
    (source/main.cpp:381-474): a .prof frame when Time + 1e-5 Dt passes
    OutputNext (before the step), a .vtk frame when it passes VtkOutputNext
    (after the solve), both numbered by the step count iStep = (int)(Time/Dt),
    and the initial output.vtk (main.cpp:374)."""
    names, log = ["output.vtk"], []
    t = time0
    step = int(t / dt)
    onext = vnext = t
    while t < end + 1.0e-5 * dt:
        if t + 1.0e-5 * dt >= onext:
            names.append("prof%03d.prof" % step)
            log.append("@ Prof Output Time : %e" % t)
            onext += out_iv
        if t + 1.0e-5 * dt >= vnext:
            names.append("vtk%03d.vtk" % step)
            log.append("@ Vtk Output Time : %e" % t)
            vnext += vtk_iv
        t += dt
        step += 1
    return sorted(names), log


def vtk_sections(text: str) -> List[Tuple[str, List[str]]]:
    """(header line, data lines) of a legacy ASCII .vtk frame, in order."""
    keys = ("POINTS", "CELLS", "CELL_TYPES", "POINT_DATA", "SCALARS", "LOOKUP_TABLE", "VECTORS")
    out: List[Tuple[str, List[str]]] = []
    head = []
    for ln in text.splitlines():
        if ln.startswith("LOOKUP_TABLE") and out and out[-1][0].startswith("SCALARS"):
            out[-1] = (out[-1][0] + " / " + ln, out[-1][1])   # a scalar's table line joins its header
        elif ln.split(" ")[0] in keys:
            out.append((ln, []))
        elif out:
            if ln.strip():
                out[-1][1].append(ln)
        else:
            head.append(ln)
    return [("HEAD", head)] + out


def _number(t: str) -> bool:
    try:
        float(t)
        return True
    except ValueError:
        return False


def compare_frame(got: str, ref: str, float_tol: float) -> Dict[str, float]:
    """Same section order, headers, words and integer data; float data within
    float_tol of the section's largest magnitude.  Returns the largest
    relative deviation per float section."""
    def prof(text):
        ln = text.splitlines()
        return [("TIME", ln[:1]), ("HEADER", ln[1:2]), ("TYPE", [l.split()[0] for l in ln[2:]]),
                ("STATE", [" ".join(l.split()[1:]) for l in ln[2:]])]
    a, b = (vtk_sections(got), vtk_sections(ref)) if ref.lstrip().startswith("#") else (prof(got), prof(ref))
    assert [h for h, _ in a] == [h for h, _ in b], ([h for h, _ in a], [h for h, _ in b])
    dev = {}
    for (h, la), (_, lb) in zip(a, b):
        assert len(la) == len(lb), (h, len(la), len(lb))
        fa = [t for l in la for t in l.split()]
        fb = [t for l in lb for t in l.split()]
        assert len(fa) == len(fb), h
        if not all(_number(t) for t in fb) or all(("." not in t and "e" not in t) for t in fb):
            assert fa == fb, h   # words and integers: exact
            continue
        va, vb = np.array(fa, float), np.array(fb, float)
        s = float(np.max(np.abs(vb))) if vb.size else 0.0
        d = float(np.max(np.abs(va - vb))) / s if s > 0 else float(np.max(np.abs(va)))
        dev[h] = d
        assert d <= float_tol, (h, d)
    return dev
