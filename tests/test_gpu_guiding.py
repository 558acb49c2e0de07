"""The guiding-centre family on the device: TrajectoryGuiding (201) and TrajectoryGuidingScatt (202),
and the reflection of focused trajectories (ReverseMomentum negates mu only).

- FP64 kernels against the oracle trajectory by trajectory, on the problems of the golden fixtures
  (whose oracle runs are pinned bit-exact to the reference's own code) with more trajectories.
- FP32 against FP64.
- Known answers: constant perpendicular diffusion across a uniform field spreads the guiding
  centres as <y^2 + z^2> = 4 D_perp t; an equatorial proton in a dipole drifts at the gradient-drift rate
  omega = 1.5 r_L v / r^2 and keeps its radius; in the dipole the magnetic moment p_perp^2 / B
  and |p| are conserved along the orbit (PPERP_METHOD 1 integrates dp_perp/dt = p_perp/(2B) dB/dt);
  pure pitch-angle scattering relaxes <mu> as mu0 exp(-2 D0 t) with each of the reference's three
  pitch-angle schemes (Euler, Milstein, RK2).
- Shock backgrounds are refused for the guiding types (their drift needs dB/dt).
"""
import math
import os
import sys

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import capi, workloads
from spectrum_gb300 import units as U
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402

from spectrum_gb300.problem import (TRAJ_FOCUSED, TRAJ_GUIDING, TRAJ_GUIDING_DIFF, TRAJ_GUIDING_DIFF_SCATT,  # noqa: E402
                                    TRAJ_GUIDING_SCATT)


def _with_mu(pb, mu):
    pb.options[workloads.SPX_OPT_MU_METHOD] = float(mu)
    return pb


@pytest.mark.parametrize("name,problem", [
    ("guiding_dipole", lambda: make_golden._guiding_dipole(128)),
    ("guidingscatt_slab", lambda: make_golden._slab_between_mirrors(TRAJ_GUIDING_SCATT, 256, d0=0.5)),
    ("focused_slab_reflect", lambda: make_golden._slab_between_mirrors(TRAJ_FOCUSED, 256)),
    ("guidingdiff_uniform", lambda: make_golden._guiding_perp(TRAJ_GUIDING_DIFF, 256, dipole=False)),
    ("guidingdiff_dipole", lambda: make_golden._guiding_perp(TRAJ_GUIDING_DIFF, 64, dipole=True)),
    ("guidingdiffscatt_uniform", lambda: make_golden._guiding_perp(TRAJ_GUIDING_DIFF_SCATT, 256, dipole=False)),
    ("guidingscatt_milstein", lambda: _with_mu(make_golden._slab_between_mirrors(TRAJ_GUIDING_SCATT, 256, d0=0.5), 1)),
    ("guidingscatt_rk2", lambda: _with_mu(make_golden._slab_between_mirrors(TRAJ_GUIDING_SCATT, 256, d0=0.5), 2)),
])
def test_fp64_matches_oracle(built_lib, name, problem):
    pb = problem()
    res = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    ot.assert_fp64_parity(res.records[0], ref, ot.run_oracle(pb, nudge_libm=1), distros=res.distros[0])


def test_focused_reflection_keeps_p_and_flips_mu(built_lib):
    """Between two reflecting planes in a uniform field the focused momentum magnitude never changes
    and every trajectory stays inside the slab (the reversal of the whole vector would make p < 0)."""
    pb = make_golden._slab_between_mirrors(TRAJ_FOCUSED, 512)
    rec = run_problems(pb, precision=capi.SPX_FP64, record=True).records[0]
    assert np.all(rec["mom"][:, 0] > 0.0)
    np.testing.assert_allclose(rec["mom"][:, 0], rec["mom0"][:, 0], rtol=1e-12)
    assert np.all(np.abs(rec["pos"][:, 0]) <= 1.0 + 0.1)


def _dipole_bmag(pos, b_eq, r_e):
    r = np.linalg.norm(pos, axis=1)
    cos_t = pos[:, 2] / r
    return b_eq * (r_e / r) ** 3 * np.sqrt(1.0 + 3.0 * cos_t ** 2)


@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_dipole_invariants(built_lib, precision):
    pb = make_golden._guiding_dipole(512)
    rec = run_problems(pb, precision=precision, record=True).records[0]
    ok = (rec["status"] & 0x10000) == 0
    r_e = workloads.R_EARTH_CM / U.unit_length
    b_eq = workloads.B_EARTH_G / U.unit_magnetic
    p0 = np.linalg.norm(rec["mom0"], axis=1)
    p1 = np.linalg.norm(rec["mom"], axis=1)
    # trajectories that stayed in the field (not lost at the Earth) over the whole time
    alive = ok & (np.linalg.norm(rec["pos"], axis=1) > 1.5 * r_e)
    assert alive.mean() > 0.8
    dp = np.abs(p1[alive] / p0[alive] - 1.0)
    assert np.median(dp) < 1e-3 and dp.max() < 2e-2, (np.median(dp), dp.max())
    mu0 = rec["mom0"][:, 0] ** 2 / _dipole_bmag(rec["pos0"], b_eq, r_e)
    mu1 = rec["mom"][:, 0] ** 2 / _dipole_bmag(rec["pos"], b_eq, r_e)
    keep = alive & (rec["mom0"][:, 0] > 0.05 * p0)
    dmu = np.abs(mu1[keep] / mu0[keep] - 1.0)
    assert np.median(dmu) < 1e-3 and dmu.max() < 5e-2, (np.median(dmu), dmu.max())


def _equatorial(t_end_s: float, n_traj: int = 8):
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundDipole, BoundaryTimeExpire, DistributionTimeUniform,
                                        InitialMomentumRing, InitialSpaceFixed, InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, Problem, distro_header
    r_e = workloads.R_EARTH_CM / U.unit_length
    b_eq = workloads.B_EARTH_G / U.unit_magnetic
    pb = Problem(traj=TRAJ_GUIDING, time_flow=FORWARD, rk=25, seed=41, n_traj=n_traj)
    c = DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
    pb.AddBackground(BackgroundDipole(), c.double(r_e).double(0.1))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0)))
    pb.AddInitial(InitialMomentumRing(), DC().double(U.mev_to_mom(10.0)).double(0.5 * math.pi))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(t_end_s / U.unit_time))
    c = distro_header(DC(), (4, 0, 0), (0.0, 0, 0), (1.0e9, 0, 0))
    pb.AddDistribution(DistributionTimeUniform(), c.double(1.0).double(0.0).int(1))
    return pb, r_e, b_eq


@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_equatorial_gradient_drift_rate(built_lib, precision):
    pb, r_e, b_eq = _equatorial(20.0)
    rec = run_problems(pb, precision=precision, record=True).records[0]
    r = 4.0 * r_e
    p = U.mev_to_mom(10.0)
    omega = 1.5 * U.LarmorRadius(p, b_eq / 64.0) * U.Vel(p) / r ** 2
    t = rec["t"]
    phi = np.abs(np.arctan2(rec["pos"][:, 1], rec["pos"][:, 0]))
    np.testing.assert_allclose(phi, omega * t, rtol=2e-3)
    np.testing.assert_allclose(np.linalg.norm(rec["pos"], axis=1), r, rtol=1e-4)
    assert np.all(np.abs(rec["pos"][:, 2]) < 1e-6 * r)


@pytest.mark.parametrize("mu_method", [0, 1, 2])
@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_guiding_scatt_isotropisation(built_lib, precision, mu_method):
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundUniform, BoundaryTimeExpire, DiffusionIsotropicConstant,
                                        DistributionTimeUniform, InitialMomentumRing, InitialSpaceFixed,
                                        InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, Problem, distro_header
    d0, t_end, theta0 = 1.0, 0.25, 0.3
    pb = Problem(traj=TRAJ_GUIDING_SCATT, time_flow=FORWARD, rk=25, seed=78, n_traj=40_000)
    pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0)).double(1.0e3))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumRing(), DC().double(1.0).double(theta0))
    pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(d0))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(t_end))
    c = distro_header(DC(), (4, 0, 0), (0.0, 0, 0), (1.0, 0, 0))
    pb.AddDistribution(DistributionTimeUniform(), c.double(1.0).double(0.0).int(1))
    pb.options[workloads.SPX_OPT_MU_METHOD] = float(mu_method)  # Euler, Milstein, RK2
    rec = run_problems(pb, precision=precision, record=True).records[0]
    p = np.linalg.norm(rec["mom"], axis=1)
    mu = rec["mom"][:, 2] / p
    expect = math.cos(theta0) * math.exp(-2.0 * d0 * rec["t"].mean())
    sigma = mu.std() / math.sqrt(len(mu))
    assert abs(mu.mean() - expect) < 4.0 * sigma + 0.01, (mu.mean(), expect)
    # |p| is rebuilt from p and mu at every scattering step: rounding accumulates (float-float
    # positions do not help the momentum, which the FP32 kernel keeps in float)
    np.testing.assert_allclose(p, 1.0, rtol=1e-10 if precision == capi.SPX_FP64 else 1e-4)
    assert np.all(rec["mom"][:, 0] >= 0.0)


def test_guiding_refuses_shock_backgrounds(built_lib):
    pb = workloads.shock_acceleration(n_traj=4)
    bg = [e for e in pb.plugins if e.plugin.role == 0][0]
    ctx = capi.Context(TRAJ_GUIDING, 0, 25, capi.SPX_FP64)
    try:
        with pytest.raises(capi.SpxError) as e:
            ctx.add_plugin(0, bg.plugin.kind, bg.blob, bg.n_records)
        assert e.value.code == -2
    finally:
        ctx.close()


def test_guiding_scatt_needs_diffusion(built_lib):
    pb = make_golden._slab_between_mirrors(TRAJ_GUIDING_SCATT, 4, d0=0.0)  # no diffusion plugin
    ctx = capi.Context(TRAJ_GUIDING_SCATT, 0, 25, capi.SPX_FP64)
    try:
        for e in pb.plugins:
            ctx.add_plugin(e.plugin.role, e.plugin.kind, e.blob, e.n_records)
        with pytest.raises(capi.SpxError) as e:
            ctx.add_problem(4, 1)
        assert e.value.code == -4
    finally:
        ctx.close()


@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_perpendicular_spread(built_lib, precision):
    pb = make_golden._guiding_perp(TRAJ_GUIDING_DIFF, 20_000, dipole=False)  # D_perp = 0.05, B along x, t = 2
    rec = run_problems(pb, precision=precision, record=True).records[0]
    r2 = rec["pos"][:, 1] ** 2 + rec["pos"][:, 2] ** 2
    expect = 4.0 * 0.05 * rec["t"].mean()
    sigma = r2.std() / math.sqrt(len(r2))
    assert abs(r2.mean() - expect) < 4.0 * sigma, (r2.mean(), expect, sigma)
    np.testing.assert_allclose(np.linalg.norm(rec["mom"], axis=1), np.linalg.norm(rec["mom0"], axis=1), rtol=1e-4)

