"""The CPU oracle against the golden fixtures made by tests/golden/make_golden.py
from the reference solver's own code (one thread).

Integer outputs (sort keys, permutations, cell ranges, neighbour lists, CR
iteration counts) must be identical; floating-point outputs agree to 1e-12
relative (bit-identical on x86_64; the margin covers libm differences of other
hosts)."""
import dataclasses
import glob
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as orc
from mphimplicit_gb300 import casegen

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(f for f in glob.glob(os.path.join(HERE, "golden", "*.npz")) if not os.path.basename(f).startswith("cli_"))
TOL = 1e-12


def load_case(z):
    p = casegen.Params(**{k: (tuple(tuple(r) for r in v) if k == "interaction_ratio" else (tuple(v) if isinstance(v, list) else v))
                          for k, v in json.loads(str(z["params"])).items()})
    parts = casegen.Particles(float(z["time"]), float(z["spacing"]), z["domain_min"], z["domain_max"], z["types"], z["pos"], z["vel"])
    return int(z["dim"]), p, parts


def close(a, b, tol=TOL):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert a.shape == b.shape, (a.shape, b.shape)
    s = max(float(np.max(np.abs(b))) if b.size else 0.0, 1e-300)
    assert float(np.max(np.abs(a - b))) <= tol * s if a.size else True


def csr_mul(ptr, ind, val, x):
    out = np.zeros(len(ptr) - 1)
    for r in range(len(ptr) - 1):
        out[r] = np.dot(val[ptr[r]:ptr[r + 1]], x[ind[ptr[r]:ptr[r + 1]]])
    return out


@pytest.fixture(scope="module", params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def fixture(request, oracle_built):
    return np.load(request.param)


def test_fixtures_present():
    names = {os.path.basename(f)[:-4] for f in FIXTURES}
    assert {"dam2d", "surface2d", "cube3d", "surface3d", "sample3d"} <= names


def test_oracle_matches_reference(fixture):
    z = fixture
    dim, p, parts = load_case(z)
    o = orc.Oracle(p, parts, dim, threads=1)
    o.init()
    N = parts.count
    for n in ("Property", "ParticleIndex"):
        assert np.array_equal(o.array(n), z["init_" + n]), n
    assert np.array_equal(o.array("CellIndex")[:N], z["init_CellIndex"])
    close(o.array("VolStrainP"), z["init_VolStrainP"])
    steps = z["cr_log"].shape[0]
    for step in range(steps):
        o.step_begin()
        if step == 0:
            close(o.array("Position"), z["s1_pos_begin"])
            close(o.array("Velocity"), z["s1_vel_begin"])
        o.cellsort()
        if step == 0:
            for n in ("CellIndex", "CellParticle"):
                assert np.array_equal(o.array(n)[:N], z["s1_" + n]), n
            for n in ("ParticleIndex", "Property", "CellFluidParticleBegin", "CellFluidParticleEnd",
                      "CellWallParticleBegin", "CellWallParticleEnd"):
                assert np.array_equal(o.array(n), z["s1_" + n]), n
        o.neighbors()
        if step == 0:
            for n in ("NeighborCount", "NeighborFluidCount", "NeighborCountP", "NeighborPtr", "NeighborInd",
                      "NeighborPtrP", "NeighborIndP"):
                assert np.array_equal(o.array(n), z["s1_" + n]), n
        o.explicit()
        if step == 0:
            for n in ("DensityA", "GravityCenter", "VolStrainP", "Kappa", "PressureA", "Force", "Velocity"):
                close(o.array(n), z["s1_" + n])
        o.assemble()
        if step == 0:
            ptr, ind, val = o.array("CsrPtrA"), o.array("CsrIndA"), o.array("CsrCofA")
            assert len(val) == int(z["s1_A_nnz"][0])
            close(csr_mul(ptr, ind, val, np.ones(len(ptr) - 1)), z["s1_A_ones"])
            close(csr_mul(ptr, ind, val, z["s1_A_w"]), z["s1_A_times_w"])
            if "s1_CsrCofA" in z:
                assert np.array_equal(ptr, z["s1_CsrPtrA"]) and np.array_equal(ind, z["s1_CsrIndA"])
                close(val, z["s1_CsrCofA"])
            close(csr_mul(o.array("CsrPtrC"), o.array("CsrIndC"), o.array("CsrCofC"), z["s1_C_w"]), z["s1_C_times_w"])
            close(o.array("VectorB"), z["s1_VectorB"])
            close(o.array("VectorP"), z["s1_VectorP"])
        o.mg_build()
        if step == 0:
            lv = o.mg_levels()
            assert len(lv) == int(z["s1_mg_depth"][0])
            for L, l in enumerate(lv):
                assert list(z[f"s1_mg{L}_geom"]) == l["min"] + l["max"] + l["count"]
                close(l["cof"].sum(axis=1), z[f"s1_mg{L}_rowsum"])
                close(np.abs(l["cof"]).sum(axis=1), z[f"s1_mg{L}_abssum"])
                close(l["invd"], z[f"s1_mg{L}_invd"])
            close(o.array("InvDiagA"), z["s1_InvDiagA"])
        it = o.solve()
        assert it == int(z["cr_log"][step][0]), (step, it, z["cr_log"][step])
        st = o.solve_stats()
        for k, col in (("rr0", 1), ("rr", 2), ("rs0", 3), ("rs", 4)):   # log prints 7 digits
            assert st[k] == pytest.approx(z["cr_log"][step][col], rel=1e-6)
        if step == 0:
            close(o.array("Velocity"), z["s1_Velocity_solved"])
        if step == steps - 1:
            o.output_fields()
            for n in ("DivergenceP", "PressureP", "VirialPressureAtParticle", "Force"):
                close(o.array(n), z["out_" + n])
        o.step_end()
    for n in ("ParticleIndex", "Property"):
        assert np.array_equal(o.array(n), z["final_" + n]), n
    close(o.array("Position"), z["final_Position"])
    close(o.array("Velocity"), z["final_Velocity"])
    close(o.array("WallCenter"), z["final_WallCenter"])


def test_generator_reproduces_reference_sample():
    z = np.load(os.path.join(HERE, "golden", "sample3d.npz"))
    b = json.loads(str(z["boid"]))
    h = b["head"]
    parts = casegen.boid_to_particles(h["ParticleDistance"][0], h["LowerDomain"], h["UpperDomain"], b["cuboids"])
    assert hashlib.sha256(casegen.generator_text(parts).encode()).hexdigest() == str(z["grid_sha256"])
    assert np.array_equal(parts.types, z["types"]) and np.array_equal(parts.pos, z["pos"])


def test_oracle_tolerance_only_moves_the_stop_test(oracle_built):
    """The oracle's stop-test constant (main.cpp:4346, rr/rr0 < 1e-12) is a
    parameter: 1e-6 (the default) gives the reference's iterates; 1e-12
    continues the same iteration further, so its solution solves the same
    system to a relative residual below 1e-12."""
    p, parts = casegen.square_drop_2d(scale=0.1, seed=0)
    runs = {}
    for tol in (None, 1e-6, 1e-12):
        o = orc.Oracle(p, parts, 2, threads=1)
        o.init()
        if tol is not None:
            o.set_tolerance(tol)
        o.step_begin(); o.cellsort(); o.neighbors(); o.explicit(); o.assemble(); o.mg_build(); o.solve()
        x = o.array("Velocity").reshape(-1, 3)
        nf = int(o.scalars()["FluidParticleEnd"])
        ptr, ind, val, b = o.array("CsrPtrA"), o.array("CsrIndA"), o.array("CsrCofA"), o.array("VectorB")
        r = b - csr_mul(ptr, ind, val, x[:nf].ravel())
        runs[tol] = (o.solve_stats(), x, float(np.linalg.norm(r) / np.linalg.norm(b)))
    assert runs[None][0] == runs[1e-6][0]
    assert np.array_equal(runs[None][1], runs[1e-6][1])
    assert runs[1e-12][0]["iter"] > runs[1e-6][0]["iter"]
    assert runs[1e-12][0]["rr"] / runs[1e-12][0]["rr0"] < 1e-24
    assert runs[1e-12][2] < 1e-12 < runs[1e-6][2] * 1e-3
