"""The two assembly kernels of A agree, and the cell-block kernel matches
the oracle on cases large enough for it to apply (at least 3 neighbour cells
of fluid along every axis).

k_assemble_cells gathers C Lambda C^T column by column through the
transposed P-lists; k_matrix_a merge-joins the P-lists pair by pair
(multiplyMatrixC, main.cpp:2590-2641).  Both sum the same products in
different orders, so they agree to rounding."""
import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine
from mphimplicit_gb300.cabi import PRECISION_MIXED
from parity_util import csr_blocks_oracle, mg_proj, rel, vec_proj

pytestmark = pytest.mark.gpu


def medium_cases():
    p2, parts2 = casegen.square_drop_2d(scale=0.25, seed=2)
    parts3 = casegen.dam_case(3, (11, 10, 12), (16, 13, 14), 0.005, seed=4,
                              fluid_types=(np.arange(11 * 10 * 12) % 4 == 0).astype(np.int32))
    p3 = casegen.baseline_params(3, 0.005, 5.0e-5)
    p3.density = (1000.0, 1100.0, 1000.0, 1000.0)
    p3.shear_viscosity = (0.1, 0.5, 0.1, 0.1)
    return [("dam2d_25", 2, p2, parts2), ("cube3d_11", 3, p3, parts3)]


CASES = medium_cases()
IDS = [c[0] for c in CASES]


def _assembled(params, parts, dim, cell):
    g = engine.Case(params, parts, dim)
    g.set_option("cell_assembly", 1 if cell else 0)
    for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build"):
        g.stage(st)
    return g


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_cell_and_row_assembly_agree(engine_lib, case):
    name, dim, params, parts = case
    a = _assembled(params, parts, dim, True)
    b = _assembled(params, parts, dim, False)
    assert np.array_equal(a.export("CsrIndA"), b.export("CsrIndA"))
    assert rel(a.export("CsrCofA"), b.export("CsrCofA")) <= 1e-12
    assert rel(a.export("VectorB"), b.export("VectorB")) <= 1e-12
    assert rel(a.export("InvDiagA"), b.export("InvDiagA")) <= 1e-12
    depth = int(a.scalars()["MultiGridDepth"])
    assert depth >= 2
    for L in range(depth):
        assert rel(a.export(f"MultiGridCsrCofA:{L}"), b.export(f"MultiGridCsrCofA:{L}")) <= 1e-12, L


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_cell_assembly_matches_oracle(engine_lib, oracle_built, case):
    name, dim, params, parts = case
    o = oracle_built.Oracle(params, parts, dim, threads=1)
    o.init()
    o.step_begin(); o.cellsort(); o.neighbors(); o.explicit(); o.assemble(); o.mg_build()
    g = _assembled(params, parts, dim, True)
    nf = g.fluid_count
    nfc = o.array("NeighborFluidCount")[:nf]
    oa = csr_blocks_oracle(o.array("CsrPtrA"), o.array("CsrCofA"), nf, nfc, dim)
    assert rel(g.export("CsrCofA"), oa) <= 1e-11
    assert rel(g.export("VectorB"), vec_proj(o.array("VectorB"), dim).ravel()) <= 1e-11
    for L, lv in enumerate(o.mg_levels()):
        assert rel(g.export(f"MultiGridCsrCofA:{L}"), mg_proj(lv["cof"], dim)) <= 1e-11, L
    # one full solve on top: same tolerance band as the other parity tests
    o.solve()
    g.stage("solve")
    vo = vec_proj(o.array("Velocity"), dim)[:nf]
    vg = vec_proj(g.export("Velocity"), dim)[:nf]
    assert np.linalg.norm(vg - vo) / np.linalg.norm(vo) <= 2e-5


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_fp32_cell_assembly_of_the_factored_form(engine_lib, case):
    """Mixed form with the factored FP64 operator: the FP32 cell-block kernel
    (blocks from the FP32 pair terms) against the FP64 cell-block kernel, and
    one full mixed solve against the FP64 form's velocity."""
    name, dim, params, parts = case
    a = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    a.set_option("inner_blocks", 1)   # keep the FP32 blocks to compare them
    a.set_option("mg_depth", 0)       # and the multigrid levels
    b = _assembled(params, parts, dim, True)
    for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build"):
        a.stage(st)
    assert np.array_equal(a.export("CsrIndA"), b.export("CsrIndA"))
    assert rel(a.export("CsrCofA"), b.export("CsrCofA")) <= 1e-6
    assert rel(a.export("VectorB"), b.export("VectorB")) <= 1e-12
    assert rel(a.export("InvDiagA"), b.export("InvDiagA")) <= 1e-6
    for L in range(int(a.scalars()["MultiGridDepth"])):
        assert rel(a.export(f"MultiGridCsrCofA:{L}"), b.export(f"MultiGridCsrCofA:{L}")) <= 1e-6, L
    a.stage("solve")
    b.stage("solve")
    assert a.solve_stats()["status"] == 0
    nf = a.fluid_count
    va = vec_proj(a.export("Velocity"), dim)[:nf]
    vb = vec_proj(b.export("Velocity"), dim)[:nf]
    assert np.linalg.norm(va - vb) / np.linalg.norm(vb) <= 2e-5


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_pair_term_inner_operator_solves(engine_lib, case):
    """The mixed form with its inner SpMV on the FP32 pair terms (no blocks),
    refined to 1e-10, reaches the FP64 form's velocity solved to 1e-12."""
    name, dim, params, parts = case
    a = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    a.set_option("inner_blocks", 0)
    a.set_solver(1e-10, 1e-3, 50)
    b = engine.Case(params, parts, dim)
    b.set_solver(1e-12, 1e-3, 50)
    a.step(1)
    b.step(1)
    assert a.solve_stats()["status"] == 0
    nf = a.fluid_count
    va = vec_proj(a.export("Velocity"), dim)[:nf]
    vb = vec_proj(b.export("Velocity"), dim)[:nf]
    assert np.linalg.norm(va - vb) / np.linalg.norm(vb) <= 1e-8


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sliced_pair_terms_match_blocks(engine_lib, case):
    """The inner operator on the sliced pair terms (g = sqrt(f) e, sliced
    P-lists and transposed P-lists) is the FP32 block operator in another
    storage: same block columns, the same D^-1 and multigrid levels (built
    without blocks on the pair path), and a solve with either takes about the same
    iterations to the same velocity (both are FP32 roundings of one operator,
    the outer residual is FP64).  The reference's tolerance 1e-6: the factored
    form, which the pair terms need, is not used far below it."""
    name, dim, params, parts = case
    cs = {}
    for blocks in (1, 0):
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_option("inner_blocks", blocks)
        g.set_option("mg_depth", 0)   # the multigrid-preconditioned form, whose levels are compared
        for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build"):
            g.stage(st)
        cols = g.export("CsrIndA")
        mg = [g.export("InvDiagA")] + [g.export(f"MultiGridCsrCofA:{L}") for L in range(int(g.scalars()["MultiGridDepth"]))]
        g.stage("solve")
        assert g.solve_stats()["status"] == 0
        cs[blocks] = (g, cols, mg)
    (a, ia, ma), (b, ib, mb) = cs[0], cs[1]
    assert np.array_equal(ia, ib)
    # D^-1 and the multigrid levels: from the pair terms (k_part_pairs) and
    # from the FP32 blocks, FP32 sums in different orders
    assert len(ma) == len(mb)
    for L, (x, y) in enumerate(zip(ma, mb)):
        assert rel(x, y) <= 1e-6, L
    sa, sb = a.solve_stats(), b.solve_stats()
    assert (sa["inner_form"], sb["inner_form"]) == (2, 1)
    # every row block of the pair-term operator is accounted for; compact
    # particle orderings stage their neighbours in shared memory
    nblk = (a.fluid_count + 511) // 512
    assert sa["inner_local_blocks"] + sa["inner_gather_blocks"] == nblk
    assert sa["inner_local_blocks"] > 0 and sa["inner_local_cols"] >= sa["inner_local_blocks"]
    assert sb["inner_local_blocks"] == sb["inner_gather_blocks"] == 0
    assert sa["inner_ct_local_blocks"] > 0
    assert abs(sa["iter"] - sb["iter"]) <= max(2, sb["iter"] // 10), (sa, sb)
    assert abs(sa["outer"] - sb["outer"]) <= 1
    nf = a.fluid_count
    va = vec_proj(a.export("Velocity"), dim)[:nf]
    vb = vec_proj(b.export("Velocity"), dim)[:nf]
    assert np.linalg.norm(va - vb) / np.linalg.norm(vb) <= 1e-5


# slot-record formats of the pair-term operator: FP16 records (8 bytes a
# slot), packed records (the default: 4-byte fixed-point g and a 2-byte
# index) and g evaluated from the staged positions
FORMATS = [("fp16", {"pair_pack": 0}), ("pack", {}), ("recompute", {"pair_recompute": 1})]
FIDS = [f[0] for f in FORMATS]


@pytest.mark.parametrize("fmt", FORMATS, ids=FIDS)
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_staged_and_gathered_operator_give_the_same_bits(engine_lib, case, fmt):
    """The pair-term operator sums the same terms in the same order whether a
    block reads its neighbours' s from its shared-memory copy or gathers it
    by column (option inner_local 0), so whole mixed steps agree bit for
    bit, in every slot-record format."""
    name, dim, params, parts = case
    out = {}
    for local in (1, 0):
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        for k, v in fmt[1].items():
            g.set_option(k, v)
        g.set_option("inner_local", local)
        g.step(2)
        st = g.solve_stats()
        assert st["inner_form"] == 2
        out[local] = (g.export("Velocity"), g.export("Position"), st)
    (va, pa, sa), (vb, pb, sb) = out[1], out[0]
    assert sa["inner_local_blocks"] > 0 and sb["inner_local_blocks"] == 0 and sb["inner_ct_local_blocks"] == 0
    assert sa["iter"] == sb["iter"]
    assert np.array_equal(va, vb) and np.array_equal(pa, pb)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_slot_record_formats_reach_the_same_solution(engine_lib, case):
    """The three slot-record formats are FP32 (or finer) roundings of one
    operator used only inside the refinement: refined to 1e-10, their
    velocities agree to about that, and their iteration counts stay close."""
    name, dim, params, parts = case
    res = {}
    for fid, opts in FORMATS:
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_solver(1e-10, 1e-3, 50)
        for k, v in opts.items():
            g.set_option(k, v)
        g.step(1)
        st = g.solve_stats()
        assert st["status"] == 0 and st["inner_form"] == 2, (fid, st)
        res[fid] = (vec_proj(g.export("Velocity"), dim)[:g.fluid_count], st["iter"])
    v0, it0 = res["fp16"]
    for fid in ("pack", "recompute"):
        v, it = res[fid]
        assert np.linalg.norm(v - v0) / np.linalg.norm(v0) <= 1e-8, fid
        assert abs(it - it0) <= max(3, it0 // 10), (fid, it, it0)


@pytest.mark.parametrize("fmt", FORMATS, ids=FIDS)
def test_mixed_staged_and_gathering_blocks_give_the_same_bits(engine_lib, fmt):
    """A case where some row blocks of the pair-term operator have more
    distinct neighbours than one block may stage (RadiusV = 7 l0: about 1400
    neighbours a particle, over 8192 distinct ones for a row block inside
    the 30^3 fluid), so the staged kernel variant meets blocks that
    gather by column (and transposed P-lists that keep their columns): its
    steps agree bit for bit with every block gathering (option inner_local
    0), in every slot-record format."""
    from mphimplicit_gb300 import casegen
    parts = casegen.dam_case(3, (30, 30, 30), (36, 34, 34), 0.005, seed=2)
    params = casegen.baseline_params(3, 0.005, 5.0e-5)
    params.radius_ratio_v = 7.0
    out = {}
    for local in (1, 0):
        g = engine.Case(params, parts, 3, precision=PRECISION_MIXED)
        for k, v in fmt[1].items():
            g.set_option(k, v)
        g.set_option("inner_local", local)
        g.step(2)
        st = g.solve_stats()
        assert st["inner_form"] == 2
        out[local] = (g.export("Velocity"), g.export("Position"), st)
    (va, pa, sa), (vb, pb, sb) = out[1], out[0]
    print(f"{fmt[0]}: staged {sa['inner_local_blocks']}, gathering {sa['inner_gather_blocks']} row blocks")
    assert sa["inner_local_blocks"] > 0 and sa["inner_gather_blocks"] > 0
    assert sa["iter"] == sb["iter"]
    assert np.array_equal(va, vb) and np.array_equal(pa, pb)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_point_jacobi_diagonal_and_solution(engine_lib, case):
    """The point-Jacobi mixed form (the default, option mg_depth -1) takes D^-1
    from the pair-term kernel instead of the level-0 pass: the same FP32 sums
    of the diagonal in another order (rel 1e-6), no multigrid levels, and a
    step refined to 1e-10 reaches the multigrid-preconditioned form's
    velocity to about that."""
    name, dim, params, parts = case
    res = {}
    for depth in (-1, 0):
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_solver(1e-10, 1e-3, 50)
        g.set_option("mg_depth", depth)
        for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build"):
            g.stage(st)
        dinv = g.export("InvDiagA")
        if depth < 0:
            with pytest.raises(engine.MphError):
                g.export("MultiGridCsrCofA:0")
        g.stage("solve")
        st = g.solve_stats()
        assert st["status"] == 0 and st["inner_form"] == 2
        res[depth] = (dinv, vec_proj(g.export("Velocity"), dim)[:g.fluid_count])
    (dj, vj), (dm, vm) = res[-1], res[0]
    assert rel(dj, dm) <= 1e-6
    assert np.linalg.norm(vj - vm) / np.linalg.norm(vm) <= 1e-8


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_fused_pair_slices_give_the_same_bits(engine_lib, case):
    """Option pair_fuse writes the sliced pair terms, the slot records and
    the slice scales in one kernel (no pair-term list) with the same pair
    evaluation and expressions as the two-kernel path: whole point-Jacobi
    mixed steps agree bit for bit except for D^-1, whose wall-slot terms it
    sums in another order (so the steps are compared to the refinement's
    tolerance, and b and the records bit for bit)."""
    name, dim, params, parts = case
    out = {}
    for fuse in (0, 1):
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_solver(1e-10, 1e-3, 50)
        g.set_option("pair_fuse", fuse)
        for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble"):
            g.stage(st)
        b, dinv = g.export("VectorB"), g.export("InvDiagA")
        g.stage("mg_build")
        g.stage("solve")
        assert g.solve_stats()["status"] == 0
        out[fuse] = (b, dinv, vec_proj(g.export("Velocity"), dim)[:g.fluid_count])
    (b0, d0, v0), (b1, d1, v1) = out[0], out[1]
    assert np.array_equal(b0, b1)
    assert rel(d1, d0) <= 1e-6
    assert np.linalg.norm(v1 - v0) / np.linalg.norm(v0) <= 1e-8
