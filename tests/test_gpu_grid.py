"""The gridded background (BackgroundServerCartesian with first-order interpolation on one block in
device memory): the FP64 kernel against the oracle trajectory by trajectory, the FP32 kernel against
FP64 and the gridded Parker spiral against its closed form, per bin within 3 sigma."""
import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import capi, workloads
from spectrum_gb300.datacontainer import DataContainer
from spectrum_gb300.plugins import BackgroundSolarWind
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu


def _within_3sigma(a, b, min_count=20):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    m = (a + b) >= min_count
    return m.sum(), np.abs(a[m] - b[m]) <= 3.0 * np.sqrt(a[m] + b[m])


@pytest.mark.parametrize("deriv_mode", [1, 0])
def test_grid_fp64_matches_oracle(built_lib, deriv_mode):
    """Trajectory by trajectory, with the analytic divergence of the diffusion tensor (1) and with
    the reference's finite-difference one (0, TRAJ_PARKER_DIVK_METHOD 0)."""
    pbs = workloads.gcr_modulation_grid(n_traj=64, n_nodes=48, energies_mev=[300.0], t_max_years=0.05)
    gpu = run_problems(pbs, precision=capi.SPX_FP64, record=True, deriv_mode=deriv_mode)
    ref = ot.run_oracle(pbs[0], deriv_mode=deriv_mode)
    ot.assert_fp64_parity(gpu.records[0], ref, ot.run_oracle(pbs[0], deriv_mode=deriv_mode, nudge_libm=1),
                          distros=gpu.distros[0])
    assert gpu.stats.given_up == 0


def test_grid_fp32_matches_fp64(built_lib):
    pbs = workloads.gcr_modulation_grid(n_traj=3000, n_nodes=96, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    r64 = run_problems(pbs, precision=capi.SPX_FP64)
    r32 = run_problems(pbs, precision=capi.SPX_MIXED)
    for k in range(len(pbs)):
        for d in range(2):
            n, ok = _within_3sigma(r32.distros[k][d][0], r64.distros[k][d][0])
            assert n >= 1 and ok.all(), (k, d)


def test_grid_spiral_matches_closed_form(built_lib):
    """The Parker spiral sampled on a 128^3 block over +-6 AU against the closed-form background
    with the same step-size rule (dmax = one zone everywhere): the exit-time histograms and the
    spectrum counts agree per bin within 3 sigma."""
    n_nodes, half = 128, 6.0
    zone = 2.0 * half * workloads.ONE_AU / (n_nodes - 1)
    kw = dict(n_traj=4000, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    grid = workloads.gcr_modulation_grid(n_nodes=n_nodes, half_width_au=half, **kw)
    closed = workloads.gcr_modulation(r_inner_au=0.3, r_outer_au=5.0, **kw)
    for pb in closed:
        c = workloads.solarwind_params(DataContainer(), dmax0=zone)
        c._records[-1] = DataContainer().double(1.0e4)._records[0]  # dmax_fraction: dmax = dmax0 everywhere
        pb.plugins[0] = type(pb.plugins[0])(BackgroundSolarWind(), c.data(), c.size())
    rg = run_problems(grid, precision=capi.SPX_MIXED)
    rc = run_problems(closed, precision=capi.SPX_MIXED)
    for k in range(len(grid)):
        for d in range(2):
            n, ok = _within_3sigma(rg.distros[k][d][0], rc.distros[k][d][0])
            assert n >= 1 and ok.mean() >= 0.95, (k, d, rg.distros[k][d][0], rc.distros[k][d][0])


@pytest.mark.parametrize("ghost,order", [(0, 1), (1, 1), (0, 0), (0, -1)])
def test_block_grid_fp64_matches_oracle(built_lib, ghost, order):
    """The reference server's block layout (spx_set_background_blocks, 12^3 blocks of 4^3 zones):
    trajectory by trajectory against the oracle, whose block-mode fields equal the reference's
    server bit for bit (test_oracle_grid_blocks.py); without and with a ghost layer per block side, and at
    SERVER_INTERP_ORDER 0 (zone values) and -1 (the reader's interpolation, numerical gradients)."""
    pbs = workloads.gcr_modulation_blocks(n_traj=64, n_blocks=12, ghost_cells=ghost, energies_mev=[300.0],
                                          t_max_years=0.05)
    pbs[0].grid.interp_order = order
    gpu = run_problems(pbs, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pbs[0])
    ot.assert_fp64_parity(gpu.records[0], ref, ot.run_oracle(pbs[0], nudge_libm=1), distros=gpu.distros[0])
    assert gpu.stats.given_up == 0


def test_block_grid_fp32_matches_fp64(built_lib):
    pbs = workloads.gcr_modulation_blocks(n_traj=3000, n_blocks=24, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    r64 = run_problems(pbs, precision=capi.SPX_FP64)
    r32 = run_problems(pbs, precision=capi.SPX_MIXED)
    for k in range(len(pbs)):
        for d in range(2):
            n, ok = _within_3sigma(r32.distros[k][d][0], r64.distros[k][d][0])
            assert n >= 1 and ok.all(), (k, d)


def test_reader_interpolation_needs_fp64(built_lib):
    """Order -1 takes numerical gradients, which only the FP64 kernels carry."""
    pbs = workloads.gcr_modulation_blocks(n_traj=10, n_blocks=2, energies_mev=[300.0])
    ctx = capi.Context(pbs[0].traj, pbs[0].time_flow, pbs[0].rk, capi.SPX_MIXED)
    try:
        with pytest.raises(capi.SpxError):
            ctx.set_option(capi.SPX_OPT_GRID_INTERP, -1.0)
        ctx.set_option(capi.SPX_OPT_GRID_INTERP, 0.0)
    finally:
        ctx.close()


def test_block_grid_rejects_bad_layouts(built_lib):
    pbs = workloads.gcr_modulation_blocks(n_traj=10, n_blocks=2, energies_mev=[300.0])
    ctx = capi.Context(pbs[0].traj, pbs[0].time_flow, pbs[0].rk, capi.SPX_MIXED)
    try:
        g = pbs[0].grid
        for nb, lo, hi, ghost in [((0, 2, 2), g.domain_min, g.domain_max, 0), (g.n_blocks, g.domain_max, g.domain_min, 0),
                                  (g.n_blocks, g.domain_min, g.domain_max, 2)]:
            with pytest.raises((capi.SpxError, ValueError)):
                ctx.set_background_blocks(nb, lo, hi, ghost, g.values)
    finally:
        ctx.close()


def test_grid_background_needs_its_grid(built_lib):
    pbs = workloads.gcr_modulation_grid(n_traj=10, n_nodes=8, energies_mev=[300.0])
    ctx = capi.Context(pbs[0].traj, pbs[0].time_flow, pbs[0].rk, capi.SPX_MIXED)
    try:
        for e in pbs[0].plugins:
            ctx.add_plugin(e.plugin.role, e.plugin.kind, e.blob, e.n_records)
        ctx.add_problem(10, 1)
        with pytest.raises(capi.SpxError) as e:
            ctx.run()
        assert e.value.code == -8  # SPX_ERR_STATE: no grid yet
        g = pbs[0].grid
        ctx.set_background_grid(g.n, g.cent_min, g.zone_length, g.values)
        ctx.run()
        assert ctx.sync().trajectories == 10
    finally:
        ctx.close()
