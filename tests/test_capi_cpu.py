"""The C-ABI library without a GPU: it loads, exports every symbol declared
in include/*.h, and its host-only entry points (file formats, argument
checks) behave like the reference's readers and writers."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from mphimplicit_gb300 import build, casegen, engine

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return engine.load_library()


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(mph_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string(lib):
    assert b"sm_103a" in lib.mph_version()
    assert lib.mph_step(None, 1) == 1            # MPH_ERR_ARG on a null handle
    assert b"null" in lib.mph_last_error()


def test_grid_and_data_roundtrip(tmp_path, lib):
    p, parts = casegen.square_drop_2d(scale=0.05, seed=7)
    p.surface_tension = (0.072, 0.0, 0.0, 0.0)
    p.wall3 = (0.1, 0.2, 0.0, 0.01, 0.0, 0.0, 0.0, 0.0, 1.5)
    d, g = casegen.write_case(str(tmp_path / "c"), p, parts)
    q = engine.read_data(d)
    assert q == p
    back = engine.read_grid(g)
    assert back.count == parts.count
    assert np.array_equal(back.types, parts.types)
    assert np.array_equal(back.pos, parts.pos) and np.array_equal(back.vel, parts.vel)
    assert np.array_equal(back.domain_min, parts.domain_min) and np.array_equal(back.domain_max, parts.domain_max)


def test_reference_data_keywords(tmp_path, lib):
    # keyword lines as in the reference's sample files (two spaces after WallN)
    txt = """#######
Dt\t\t\t\t2.0e-3
OutputInterval\t\t\t1.0
VtkOutputInterval\t\t5.0e-2
EndTime\t\t\t\t1.0
RadiusRatioA\t\t\t\t\t3.5
RadiusRatioP\t\t\t\t\t1.75
RadiusRatioV\t\t\t\t\t3.5
Density\t\t\t\t\t\t\t1.0e+3\t\t1.0e+3\t\t1.0e+3\t\t1.0e+3
BulkModulus 1e6 1e6 1e6 1e6
BulkViscosity 2e3 2e3 2e3 2e3
ShearViscosity 1e3 1e3 1e3 1e3
SurfaceTension 0 0 0 0
InteractionRatio(Type0) 1 1 1 1
InteractionRatio(Type1) 1 1 1 1
InteractionRatio(Type2) 1 1 1 1
InteractionRatio(Type3) 1 1 1 1
Gravity                         0.0 -1.0 0.0
Wall2    Center 0.0 0.0 0.0    Velocity 0.0 0.0 0.0    Omega 0.0 0.0 0.0
Wall3    Center 1.0 2.0 3.0    Velocity 4.0 5.0 6.0    Omega 7.0 8.0 9.0
Density 1 2 3
garbage line
"""
    f = tmp_path / "x.data"
    f.write_text(txt)
    q = engine.read_data(str(f))
    assert q.dt == 2.0e-3 and q.radius_ratio_p == 1.75 and q.density == (1000.0,) * 4   # 3-value line ignored
    assert q.gravity == (0.0, -1.0, 0.0)
    assert q.wall3 == (1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0)


def test_short_grid_is_an_error(tmp_path, lib):
    f = tmp_path / "short.grid"
    f.write_text("0.0\n3 0.01 0 1 0 1 0 1\n0 0.1 0.1 0 0 0 0\n")
    with pytest.raises(engine.MphError) as e:
        parts = casegen.Particles(0, 0, np.zeros(3), np.zeros(3), np.zeros(3, np.int32), np.zeros((3, 3)), np.zeros((3, 3)))
        from mphimplicit_gb300.cabi import MphParticles, np_ptr
        s = MphParticles()
        s.count = 3
        s.type = np_ptr(parts.types, ctypes.c_int)
        s.pos = np_ptr(parts.pos)
        s.vel = np_ptr(parts.vel)
        engine._check(lib.mph_read_grid(str(f).encode(), ctypes.byref(s)))
    assert e.value.status == 2
    with pytest.raises(engine.MphError):
        engine.read_grid(str(tmp_path / "missing.grid"))


def test_case_validation_without_gpu(lib):
    """Inputs the reference cannot run are refused before any device work."""
    p, parts = casegen.square_drop_2d(scale=0.05)
    bad = casegen.Particles(parts.time, parts.spacing, parts.domain_min, parts.domain_max,
                            parts.types.copy(), parts.pos.copy(), parts.vel.copy())
    bad.types[0] = 7
    with pytest.raises(engine.MphError) as e:
        engine.Case(p, bad, 2)
    assert e.value.status == 3
    bad = casegen.Particles(parts.time, parts.spacing, parts.domain_min, parts.domain_max,
                            parts.types.copy(), parts.pos.copy(), parts.vel.copy())
    bad.vel[0, 2] = 1.0   # a z velocity in a 2D case
    with pytest.raises(engine.MphError) as e:
        engine.Case(p, bad, 2)
    assert e.value.status == 3
    with pytest.raises(engine.MphError) as e:
        engine.Case(p, parts, 4)
    assert e.value.status == 1


def test_footprint_bound_scales_with_case(lib):
    from mphimplicit_gb300 import serving
    from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
    p1, s1 = casegen.square_drop_2d(scale=0.1, seed=0)
    p2, s2 = casegen.square_drop_2d(scale=0.3, seed=0)
    a = serving.footprint(p1, s1, 2, PRECISION_FP64)
    b = serving.footprint(p2, s2, 2, PRECISION_FP64)
    m = serving.footprint(p2, s2, 2, PRECISION_MIXED)
    assert 0 < a < b < m
    s3 = casegen.dam_case(3, (12, 12, 12), (16, 16, 16), 0.005, seed=0)
    p3 = casegen.baseline_params(3, 0.005, 5.0e-5)
    c = serving.footprint(p3, s3, 3, PRECISION_FP64)
    # beyond the fixed 64 MiB, a 3D fluid particle (its matrix row) costs
    # several times a 2D one
    fixed = 64 << 20
    assert (c - fixed) / (s3.types < 2).sum() > 3 * (b - fixed) / (s2.types < 2).sum()
    # the 3D mixed form steps on pair terms (no assembled blocks) by default,
    # so its bound is below the FP64 form's, whose FP64 blocks dominate
    assert serving.footprint(p3, s3, 3, PRECISION_MIXED) < c


def test_server_rejects_requests_beyond_budget(lib):
    from mphimplicit_gb300 import serving
    p, s = casegen.square_drop_2d(scale=0.1, seed=0)
    srv = serving.Server(budget_bytes=1 << 20, workers=1)
    with pytest.raises(engine.MphError) as e:
        srv.submit(p, s, 2, steps=1)
    assert e.value.status == 6
    with pytest.raises(engine.MphError):
        srv.submit(p, s, 2, steps=0)
    assert srv.stats()["pending"] == 0
    srv.close()


def test_checkpoint_roundtrip_is_exact(tmp_path, lib):
    rng = np.random.default_rng(7)
    p, s = casegen.square_drop_2d(scale=0.1, seed=0)
    s = casegen.Particles(1.25e-3, s.spacing, s.domain_min, s.domain_max, s.types,
                          s.pos + rng.uniform(-1e-9, 1e-9, s.pos.shape), rng.standard_normal(s.vel.shape))
    ids = rng.permutation(len(s.types)).astype(np.int32)
    wc = rng.standard_normal((4, 3))
    path = str(tmp_path / "state.ckpt")
    engine.write_checkpoint(path, s, ids, wc)
    r, rid, rwc = engine.read_checkpoint(path)
    assert r.time == s.time and r.spacing == s.spacing
    assert np.array_equal(r.domain_min, s.domain_min) and np.array_equal(r.domain_max, s.domain_max)
    assert np.array_equal(r.types, s.types) and np.array_equal(rid, ids)
    assert np.array_equal(r.pos, s.pos) and np.array_equal(r.vel, s.vel) and np.array_equal(rwc, wc)


def test_checkpoint_rejects_other_files(tmp_path, lib):
    bad = tmp_path / "box.grid"
    bad.write_text("0.0\n0.01\n")
    with pytest.raises(engine.MphError) as e:
        engine.read_checkpoint(str(bad))
    assert e.value.status == 2
