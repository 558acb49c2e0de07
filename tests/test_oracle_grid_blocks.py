"""The gridded background in block mode against the reference's own Cartesian data server: its
reader, blocks and front end (src/reader_cartesian.cc, src/block_base.cc, src/server_cartesian.cc)
compiled here through a stand-in MPI header and driven on one process by
oracle/ref_glue/grid_harness.cc. Every field and gradient is compared bit for bit with the oracle's
restatement at points inside blocks, next to block faces (plane stencils) and next to block edges
and corners (stencils over several blocks). The golden fixture (tests/golden/grid_blocks_ref.npz,
written by make_golden.py from the same harness) keeps the comparison where the reference is absent."""
import os
import subprocess

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300.problem import BlockGrid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
GOLDEN = os.path.join(ROOT, "tests", "golden", "grid_blocks_ref.npz")
AU = 1.495978707e13
L = 1.0e10


def _harness(ghost, variant=""):
    exe = os.path.join(REF, f"ref_grid{ghost}{variant}")
    if not os.path.exists(exe):
        pytest.skip("the reference's grid harness is not built here (make -C oracle grid-ref)")
    return exe


def synthetic_grid(ghost=0, seed=3):
    """3 x 3 x 2 blocks over an off-centre box, random fluid-unit fields with a strong B."""
    rng = np.random.default_rng(seed)
    nb, lo, hi = (3, 3, 2), (-1.5, -1.2, -0.9), (1.5, 1.8, 0.9)
    v = rng.normal(size=(18, 64, 6))
    v[..., 3:] += (20.0, -15.0, 8.0)
    return BlockGrid(nb, lo, hi, v, ghost)


def probe_points(g, seed=4):
    """Code-unit positions whose stencils stay inside the domain: random interior points, and points
    1e-6 of a zone off every inner block face (plane stencils), edge and corner."""
    rng = np.random.default_rng(seed)
    lo, hi, nb = np.array(g.domain_min), np.array(g.domain_max), np.array(g.n_blocks)
    zl = (hi - lo) / nb / 4.0
    inner_lo, inner_hi = lo + 0.6 * zl, hi - 0.6 * zl
    pts = [inner_lo + (inner_hi - inner_lo) * rng.random(3) for _ in range(60)]
    faces = [lo[k] + (hi[k] - lo[k]) / nb[k] * np.arange(1, nb[k]) for k in range(3)]
    for sgn in (-1.0, 1.0):
        for fx in faces[0]:
            pts.append(np.array([fx + sgn * 1e-6 * zl[0], 0.13, 0.07]))
            for fy in faces[1]:
                pts.append(np.array([fx + sgn * 1e-6 * zl[0], fy - sgn * 1e-6 * zl[1], -0.21]))
                for fz in faces[2]:
                    pts.append(np.array([fx - sgn * 1e-6 * zl[0], fy + sgn * 1e-6 * zl[1], fz + sgn * 1e-6 * zl[2]]))
    return np.array(pts) * AU / L


def run_harness(ghost, g, pts, dmax0, tmp_path, variant=""):
    dat = str(tmp_path / "grid.dat")
    g.write(dat)
    text = f"{dat} {dmax0!r}\n" + "".join(" ".join(repr(float(x)) for x in p) + "\n" for p in pts)
    out = subprocess.run([_harness(ghost, variant)], input=text, capture_output=True, text=True, check=True).stdout
    return [None if line.strip() == "ERR" else line.split() for line in out.strip().split("\n")]


def test_reader_files_round_trip(tmp_path):
    g = synthetic_grid()
    g.write(str(tmp_path / "x.dat"))
    h = BlockGrid.read(str(tmp_path / "x.dat"))
    assert h.n_blocks == g.n_blocks and h.domain_min == g.domain_min and h.domain_max == g.domain_max
    assert np.array_equal(h.values, g.values)


def test_grid_units_equal_the_reference(built_lib):
    """The unit ratios of the oracle, of the library (spx_grid_units, no device needed) and of the
    workload builder are the reference's doubles."""
    from spectrum_gb300 import capi, workloads
    out = subprocess.run([_harness(0)], input="units\n", capture_output=True, text=True, check=True).stdout
    ref = np.array([float(x) for x in out.split()])
    assert np.array_equal(ot.grid_units(), ref)
    assert np.array_equal(capi.grid_units(), ref)
    assert np.array_equal(np.array(workloads.server_unit_ratios()), ref)


def test_block_fields_equal_the_reference(tmp_path):
    """GetVariables + GetGradients of the front end (every block cached, no ghost cells): the oracle's
    block mode gives the same doubles, including the plane (status 1-3) and edge/corner (status 4)
    stencils that take zones from neighbouring blocks."""
    g = synthetic_grid()
    pts = probe_points(g)
    dmax0 = 0.05 * AU / L
    rows = run_harness(0, g, pts, dmax0, tmp_path)
    ot.set_grid(g)
    statuses = set()
    for p, row in zip(pts, rows):
        assert row is not None, p
        statuses.add(int(row[0]))
        ref = np.array([float(x) for x in row[1:]])
        mine = ot.grid_fields(p, dmax0)
        assert mine is not None, p
        assert np.array_equal(mine, ref), (p, np.flatnonzero(mine != ref), mine - ref)
    assert {0, 1, 2, 4} <= statuses  # interior, planes in x and y, edges and corners


@pytest.mark.parametrize("order,variant", [(0, "_order0"), (-1, "_reader")])
def test_other_orders_equal_the_reference(tmp_path, order, variant):
    """SERVER_INTERP_ORDER 0 (the values of the zone holding the point, zero gradients) and -1 (the boss's
    reader interpolation over the whole domain, played in process by the harness): U, B, |B|, E and dmax
    equal the oracle's bit for bit, and order 0's gradients are zero in both. (Order -1's gradients are
    the background's numerical derivatives, the routine pinned for the analytic backgrounds.)"""
    g = synthetic_grid()
    g.interp_order = order
    pts = probe_points(g)
    dmax0 = 0.05 * AU / L
    rows = run_harness(0, g, pts, dmax0, tmp_path, variant)
    ot.set_grid(g)
    for p, row in zip(pts, rows):
        assert row is not None, p
        ref = np.array([float(x) for x in row[1:]])
        mine = ot.grid_fields(p, dmax0)
        assert mine is not None, p
        n = 11 if order == -1 else 32  # U B Bmag E dmax; order 0 also its (zero) gradients
        assert np.array_equal(mine[:n], ref[:n]), (p, np.flatnonzero(mine[:n] != ref[:n]))


def test_ghost_cell_geometry_equals_the_reference(tmp_path):
    """With one ghost layer per block side the block grows by a zone each way and the stencil's
    origin, zone length, offsets, weights and derivative weights move with it (BlockBase::SetGhostCells,
    LoadDimensions); the oracle's geometry is the reference's, bit for bit. (The reference's reader
    fills no ghost zones, so only the geometry is compared.)"""
    g = synthetic_grid(ghost=1)
    pts = probe_points(g)
    rows = run_harness(1, g, pts, 1.0, tmp_path)
    ot.set_grid(g)
    nb = g.n_blocks
    for p, row in zip(pts, rows):
        assert row is not None, p
        st = ot.grid_stencil(p)
        assert st is not None, p
        node = int(row[0])
        assert node == st["node"][0] + nb[0] * (st["node"][1] + nb[1] * st["node"][2])
        vals = [float(x) for x in row[1:7]]
        assert np.array_equal(st["cent_min"], vals[:3]) and np.array_equal(st["zone_length"], vals[3:6])
        assert list(st["zone"]) == [int(x) for x in row[7:10]]
        assert np.array_equal(st["offset"], [float(x) for x in row[10:13]])
        assert np.array_equal(st["weights"], [float(x) for x in row[13:21]])
        assert np.array_equal(st["derivs"], [float(x) for x in row[21:45]])


def test_block_fields_equal_the_golden_fixture():
    """The same comparison against the fixture make_golden.py wrote from the harness."""
    if not os.path.exists(GOLDEN):
        pytest.skip("no golden fixture")
    f = np.load(GOLDEN)
    g = BlockGrid(tuple(int(x) for x in f["n_blocks"]), tuple(f["domain_min"]), tuple(f["domain_max"]), f["values"], 0)
    ot.set_grid(g)
    for p, ref in zip(f["points"], f["fields"]):
        mine = ot.grid_fields(p, float(f["dmax0"]))
        assert mine is not None and np.array_equal(mine, ref), p
