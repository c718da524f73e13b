"""Generate the golden fixtures of tests/golden/ from the reference solver.

Runs the reference's own code (MphImplicit source/main.cpp compiled with
oracle/ref_harness.cpp into oracle/_ref/, one OpenMP thread) on small seeded
cases, stage by stage, and stores inputs and outputs as compressed .npz
files.  Large matrices are stored as products with fixed vectors (A*1, A*w),
which pins every coefficient row by row without storing the matrix.

Also records the reference's own 3D sample case (results3d/.../box.grid,
box.data) and its generator input (box.boid), so the case generator can be
checked against the reference pre-processor byte for byte.

Also runs the reference executables themselves (main() and its time loop,
compiled into oracle/_ref/Mph_gcc and Mph_gcc3d) on a short 2D and 3D case
with chosen output intervals, and stores their input files, every .prof and
.vtk frame they write (output.vtk included) and the output lines of their
log: the fixtures of the command-line and frame-writer parity tests.

Run in the development container (needs the reference checkout):
    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py cli        # the executable fixtures only
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")]
os.environ["OMP_NUM_THREADS"] = "1"

import oracle as orc  # noqa: E402
from mphimplicit_gb300 import casegen  # noqa: E402
from parity_util import small_cases  # noqa: E402

REF_ROOT = "/root/reference"
SAMPLE3D = os.path.join(REF_ROOT, "results3d", "Cube_rv35_rp17_lX02_dtZ01_gX01_muX01")
STEPS = 3


def csr_mul(ptr, ind, val, x):
    out = np.zeros(len(ptr) - 1)
    for r in range(len(ptr) - 1):
        a, b = ptr[r], ptr[r + 1]
        out[r] = np.dot(val[a:b], x[ind[a:b]])
    return out


def params_json(p: casegen.Params) -> str:
    import dataclasses
    return json.dumps(dataclasses.asdict(p))


def run_case(name, dim, params, parts, store_full_a=False):
    r = orc.Reference(params, parts, dim)
    out = {"name": name, "dim": dim, "params": params_json(params), "count": parts.count,
           "time": parts.time, "spacing": parts.spacing, "domain_min": parts.domain_min, "domain_max": parts.domain_max,
           "types": parts.types, "pos": parts.pos, "vel": parts.vel}
    N = parts.count
    for n in ("Property", "ParticleIndex", "VolStrainP", "DensityA"):
        out["init_" + n] = r.array(n)
    out["init_CellIndex"] = r.array("CellIndex")[:N]
    rng = np.random.default_rng(1234)
    log_iters = []
    for step in range(STEPS):
        r.step_begin()
        if step == 0:
            out["s1_pos_begin"] = r.array("Position")
            out["s1_vel_begin"] = r.array("Velocity")
        r.cellsort()
        if step == 0:
            for n in ("CellIndex", "CellParticle"):
                out["s1_" + n] = r.array(n)[:N]
            for n in ("ParticleIndex", "Property", "CellFluidParticleBegin", "CellFluidParticleEnd",
                      "CellWallParticleBegin", "CellWallParticleEnd"):
                out["s1_" + n] = r.array(n)
        r.neighbors()
        if step == 0:
            for n in ("NeighborCount", "NeighborFluidCount", "NeighborCountP", "NeighborPtr", "NeighborInd",
                      "NeighborPtrP", "NeighborIndP"):
                out["s1_" + n] = r.array(n)
        r.explicit()
        if step == 0:
            for n in ("DensityA", "GravityCenter", "VolStrainP", "Kappa", "PressureA", "Force", "Velocity"):
                out["s1_" + n] = r.array(n)
        r.assemble()
        if step == 0:
            ptr, ind, val = r.array("CsrPtrA"), r.array("CsrIndA"), r.array("CsrCofA")
            ncol = len(ptr) - 1
            w = rng.standard_normal(ncol)
            out["s1_A_w"] = w
            out["s1_A_ones"] = csr_mul(ptr, ind, val, np.ones(ncol))
            out["s1_A_times_w"] = csr_mul(ptr, ind, val, w)
            out["s1_A_nnz"] = np.array([len(val)])
            if store_full_a:
                out["s1_CsrPtrA"], out["s1_CsrIndA"], out["s1_CsrCofA"] = ptr, ind, val
            cptr, cind, cval = r.array("CsrPtrC"), r.array("CsrIndC"), r.array("CsrCofC")
            wc = rng.standard_normal(N)
            out["s1_C_w"] = wc
            out["s1_C_times_w"] = csr_mul(cptr, cind, cval, wc)
            out["s1_VectorB"] = r.array("VectorB")
            out["s1_VectorP"] = r.array("VectorP")
        r.free_c()
        r.mg_build()
        if step == 0:
            lv = r.mg_levels()
            out["s1_mg_depth"] = np.array([len(lv)])
            for L, l in enumerate(lv):
                out[f"s1_mg{L}_geom"] = np.array(l["min"] + l["max"] + l["count"])
                out[f"s1_mg{L}_rowsum"] = np.add.reduceat(l["cof"], l["ptr"][:-1]) if len(l["cof"]) else np.zeros(0)
                out[f"s1_mg{L}_abssum"] = np.add.reduceat(np.abs(l["cof"]), l["ptr"][:-1]) if len(l["cof"]) else np.zeros(0)
                out[f"s1_mg{L}_invd"] = l["invd"]
            out["s1_InvDiagA"] = r.array("InvDiagA")
        r.solve()
        log_iters.append(r.solve_log()[-1])
        if step == 0:
            out["s1_Velocity_solved"] = r.array("Velocity")
        if step == STEPS - 1:
            r.output_fields()
            for n in ("DivergenceP", "PressureP", "VirialPressureAtParticle", "Force"):
                out["out_" + n] = r.array(n)
        r.step_end()
    out["cr_log"] = np.array(log_iters)
    for n in ("Position", "Velocity", "ParticleIndex", "Property"):
        out["final_" + n] = r.array(n)
    out["final_WallCenter"] = r.array("WallCenter")
    return out


def parse_boid(path):
    txt = open(path).read()
    head = {}
    for key in ("ParticleDistance", "LowerDomain", "UpperDomain"):
        m = re.search(rf"^\s*{key}\s+(.+)$", txt, re.M)
        head[key] = [float(v) for v in m.group(1).split()]
    cubs = []
    for blk in re.findall(r"StartCuboid(.*?)EndCuboid", txt, re.S):
        c = {}
        for key in ("Spacing", "Type", "Lower", "Upper", "Velocity"):
            m = re.search(rf"^\s*{key}\s+(.+)$", blk, re.M)
            c[key] = [float(v) for v in m.group(1).split()]
        cubs.append({"space": c["Spacing"][0], "type": int(c["Type"][0]), "lower": c["Lower"], "upper": c["Upper"],
                     "velocity": c["Velocity"]})
    return head, cubs


def cli_cases():
    """(name, dim, params, particles) of the executable fixtures: the 2D dam
    and the 3D cube parity cases, 10 steps, a .prof frame every 3 steps and a
    .vtk frame every 4."""
    import dataclasses
    out = []
    for name, dim, p, parts in small_cases():
        if name not in ("dam2d", "cube3d"):
            continue
        q = dataclasses.replace(p, end_time=9 * p.dt, output_interval=3 * p.dt, vtk_output_interval=4 * p.dt)
        out.append((name, dim, q, parts))
    return out


def run_cli(name, dim, params, parts):
    """Run the reference executable (one thread) in a scratch directory and
    collect its inputs, frames and log output lines."""
    import subprocess
    import tempfile
    exe = os.path.join(REPO, "oracle", "_ref", "Mph_gcc" if dim == 2 else "Mph_gcc3d")
    with tempfile.TemporaryDirectory() as tmp:
        data, grid = casegen.write_case(os.path.join(tmp, "case"), params, parts)
        subprocess.run([exe, data, grid, "prof%03d.prof", "vtk%03d.vtk", "case.log", "1"], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        files = {}
        for fn in sorted(os.listdir(tmp)):
            if fn.endswith(".prof") or fn.endswith(".vtk"):
                files[fn] = open(os.path.join(tmp, fn), "rb").read()
        log = [ln for ln in open(os.path.join(tmp, "case.log")).read().splitlines() if ln.startswith("@ ")]
        inputs = {"case.data": open(data, "rb").read(), "case.grid": open(grid, "rb").read()}
    out = {"name": name, "dim": dim, "log": json.dumps(log), "names": json.dumps(sorted(files)),
           "inputs": json.dumps(sorted(inputs))}
    for k, v in files.items():
        out["file:" + k] = np.frombuffer(v, dtype=np.uint8)
    for k, v in inputs.items():
        out["input:" + k] = np.frombuffer(v, dtype=np.uint8)
    return out


def main_cli():
    orc.build_oracle(ref=True)
    for name, dim, p, parts in cli_cases():
        out = run_cli(name, dim, p, parts)
        np.savez_compressed(os.path.join(HERE, f"cli_{name}.npz"), **out)
        print("wrote", f"cli_{name}", json.loads(out["names"]))


def main():
    orc.build_oracle(ref=True)
    main_cli()
    for name, dim, p, parts in small_cases():
        out = run_case(name, dim, p, parts, store_full_a=(name == "dam2d"))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name, parts.count)
    # the reference's 3D sample case, read through the engine-independent parser
    from mphimplicit_gb300 import cabi  # noqa: F401
    head, cubs = parse_boid(os.path.join(SAMPLE3D, "box.boid"))
    grid_bytes = open(os.path.join(SAMPLE3D, "box.grid"), "rb").read()
    parts = casegen.boid_to_particles(head["ParticleDistance"][0], head["LowerDomain"], head["UpperDomain"], cubs)
    data_txt = open(os.path.join(SAMPLE3D, "box.data")).read()
    params = parse_data_text(data_txt)
    out = run_case("sample3d", 3, params, parts)
    out["boid"] = json.dumps({"head": head, "cuboids": cubs})
    out["grid_sha256"] = hashlib.sha256(grid_bytes).hexdigest()
    np.savez_compressed(os.path.join(HERE, "sample3d.npz"), **out)
    print("wrote sample3d", parts.count)


def parse_data_text(txt: str) -> casegen.Params:
    p = casegen.Params()
    vals = {}
    for line in txt.splitlines():
        f = line.split()
        if not f or f[0].startswith("#"):
            continue
        vals[f[0]] = f[1:]
    num = lambda k, n: tuple(float(v) for v in vals[k][:n])
    p.dt = num("Dt", 1)[0]
    p.output_interval = num("OutputInterval", 1)[0]
    p.vtk_output_interval = num("VtkOutputInterval", 1)[0]
    p.end_time = num("EndTime", 1)[0]
    p.radius_ratio_a = num("RadiusRatioA", 1)[0]
    p.radius_ratio_p = num("RadiusRatioP", 1)[0]
    p.radius_ratio_v = num("RadiusRatioV", 1)[0]
    p.density = num("Density", 4)
    p.bulk_modulus = num("BulkModulus", 4)
    p.bulk_viscosity = num("BulkViscosity", 4)
    p.shear_viscosity = num("ShearViscosity", 4)
    p.surface_tension = num("SurfaceTension", 4)
    p.interaction_ratio = tuple(num(f"InteractionRatio(Type{t})", 4) for t in range(4))
    p.gravity = num("Gravity", 3)
    for t, attr in ((2, "wall2"), (3, "wall3")):
        w = vals[f"Wall{t}"]
        setattr(p, attr, tuple(float(w[i]) for i in (1, 2, 3, 5, 6, 7, 9, 10, 11)))
    return p


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "cli":
        main_cli()
    else:
        main()
