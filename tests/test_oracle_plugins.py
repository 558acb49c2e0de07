"""The oracle against the reference's own code, one plugin class at a time.

The golden fixtures exercise the plugin classes the benchmark set-ups use. Here every other
boundary, initial condition, diffusion model, distribution and background class of the reference
is swapped into a small problem and run by both the C restatement and the reference's sources
(oracle/_ref, built where the sources are present): trajectories (attempts, outcome bits, steps,
initial and final state, weights) and every histogram bin must agree bit for bit. Runs on the CPU;
skipped where the reference harness is not built.
"""
import os

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import units as U
from spectrum_gb300 import workloads as W
from spectrum_gb300.datacontainer import DataContainer as DC
from spectrum_gb300.plugins import (BackgroundDipole, BackgroundShock, BackgroundSmoothShock, BackgroundSolarWind,
                                    BackgroundUniform,
                                    BoundaryBoxReflect, BoundaryCylinderAbsorb, BoundaryMomentumInjectRestrictShell,
                                    BoundaryMomentumInjectRestrictSlab, BoundaryMomentumPass, BoundaryPlanePass,
                                    BoundaryRankineAbsorb, BoundaryRegionAbsorb,
                                    BoundarySphereAbsorb, BoundarySphereReflect, BoundaryTimeExpire, BoundaryTimePass, BoundaryTimeRecurrent,
                                    DiffusionEmpiricalSOQLTandUNLT, DiffusionFlowMomentumPowerLaw, DiffusionFullConstant,
                                    DiffusionKineticEnergyRadialDistancePowerLaw, DiffusionParaConstant,
                                    DiffusionPerpConstant, DiffusionPotgieterEtAl2015, DiffusionQLTConstant,
                                    DiffusionStraussEtAl2013, DiffusionWNLTConstant, DiffusionWNLTRampVLISM,
                                    DistributionDivergenceFlowPowerLaw, DistributionMomentumUniform,
                                    DistributionPositionCumulativeOrder1, DistributionPositionCumulativeOrder2,
                                    DistributionPositionMomentumUniform, DistributionPositionUniform,
                                    DistributionSpectrumKineticEnergyBentPowerLaw, DistributionTimeUniform,
                                    InitialMomentumBeam, InitialMomentumFixed, InitialMomentumMaxwell,
                                    InitialMomentumRing, InitialMomentumShell, InitialMomentumThickShell,
                                    InitialSpaceBox, InitialSpaceCircle, InitialSpaceCylinder, InitialSpaceCylinderSector,
                                    InitialSpaceFixed, InitialSpaceLine,
                                    InitialSpaceRankineHalfBody, InitialSpaceSphere, InitialSpaceSphereSector,
                                    InitialTimeFixed, InitialTimeInterval, SourceConstant, SourceMomentumInjection,
                                    SourceSphericalShockInjection)
from spectrum_gb300.problem import (BACKWARD, FORWARD, TRAJ_FIELDLINE, TRAJ_FOCUSED, TRAJ_GUIDING, TRAJ_GUIDING_DIFF, TRAJ_GUIDING_DIFF_SCATT,
                                    TRAJ_GUIDING_SCATT, TRAJ_LORENTZ, TRAJ_PARKER,
                                    TRAJ_PARKER_SOURCE, Problem, distro_header)

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(ot.REF_DIR, "ref_guidingdiffscatt_fwd_rk25")),
                                reason="reference harness not built (needs the reference sources)")

B = W._boundary
OUTCOME = 0x01F0 | 0x10000


def _same(pb):
    # deviation D1 (the smooth shock's step limit) reproduced as the reference has it, as for the fixtures
    a, b = ot.run_oracle(pb, reference_quirks=1), ot.run_reference(pb)
    assert len(a.traj) == len(b.traj)
    for f in a.traj.dtype.names:
        if f == "status":
            assert np.array_equal(a.traj[f] & OUTCOME, b.traj[f] & OUTCOME), f
        else:
            assert np.array_equal(a.traj[f], b.traj[f]), f
    for (ca, sa, na), (cb, sb, nb) in zip(a.distros, b.distros):
        assert na == nb and np.array_equal(ca, cb) and np.array_equal(sa, sb, equal_nan=True)
    return a


def _parker(n=24, t_end=0.2, bg=None, diff=None, it=None, is_=None, im=None, dist=None, bnds=(), seed=0xFACE,
            traj=TRAJ_PARKER, flow=FORWARD, t_action=(0,), src=None):
    """Parker (or another type) in a uniform field along z, isotropic kappa = 1, dmax 0.05."""
    rk = 0 if traj in (TRAJ_PARKER, TRAJ_PARKER_SOURCE) else 25
    pb = Problem(traj=traj, time_flow=flow, rk=rk, seed=seed, n_traj=n)
    pb.AddBackground(*(bg or (BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0))
                              .double(0.05))))
    if diff is not False:
        pb.AddDiffusion(*(diff or (DiffusionFullConstant(), DC().double(1.0).double(1.0))))
    if src is not None:
        pb.AddSource(*src)
    pb.AddInitial(*(it or (InitialTimeFixed(), DC().double(0.0))))
    pb.AddInitial(*(is_ or (InitialSpaceFixed(), DC().vec((0, 0, 0)))))
    pb.AddInitial(*(im or (InitialMomentumShell(), DC().double(1.0))))
    pb.AddBoundary(BoundaryTimeExpire(), B(DC(), 1, list(t_action)).double(t_end))
    for bnd in bnds:
        pb.AddBoundary(*bnd)
    if dist is None:
        c = distro_header(DC(), (20, 0, 0), (-1.0, 0, 0), (1.0, 0, 0))
        dist = (DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(0))
    pb.AddDistribution(*dist)
    return pb


def _shock(smooth=True):
    """The diffusive-shock set-up: upstream flow 1 along x into a shock of compression 4."""
    c = DC().double(0.0).vec((0, 0, 0)).vec((1.0, 0, 0)).vec((0, 0, 1.0)).double(0.02)
    c.vec((1.0, 0, 0)).double(0.0).double(4.0)
    if smooth:
        return BackgroundSmoothShock(), c.double(0.01).double(0.1)
    return BackgroundShock(), c


# -- spatial and time boundaries -----------------------------------------------------------------
BOUNDARY_CASES = {
    "plane_pass": (BoundaryPlanePass(), B(DC(), -1, [0]).vec((0.2, 0, 0)).vec((1.0, 0, 0))),
    "sphere_reflect": (BoundarySphereReflect(), B(DC(), -1, [-1]).vec((0, 0, 0)).double(0.4)),
    "box_reflect": (BoundaryBoxReflect(), B(DC(), -1, [-1]).vec((-0.3, -0.3, -0.3)).vec((0.6, 0, 0)).vec((0, 0.6, 0))
                    .vec((0, 0, 0.6))),
    "cylinder_absorb": (BoundaryCylinderAbsorb(), B(DC(), 1, [0]).vec((0, 0, 0)).vec((0, 0, 1.0)).double(0.3)),
    "rankine_absorb": (BoundaryRankineAbsorb(), B(DC(), 1, [0]).vec((-0.4, 0, 0)).vec((1.0, 0, 0)).double(0.2)),
    "time_pass": (BoundaryTimePass(), B(DC(), -1, [0]).double(0.1)),
    "time_recurrent": (BoundaryTimeRecurrent(), B(DC(), 5, [0]).double(0.03)),
}


@pytest.mark.parametrize("name", sorted(BOUNDARY_CASES))
def test_boundary_classes(name):
    _same(_parker(bnds=[BOUNDARY_CASES[name]]))


def test_region_absorb_at_a_shock():
    """BoundaryRegionAbsorb on the shock's region indicator (upstream/downstream)."""
    pb = _parker(bg=_shock(smooth=False), bnds=[(BoundaryRegionAbsorb(), B(DC(), 1, [0]).int(0).double(1.5))],
                 is_=(InitialSpaceFixed(), DC().vec((-0.05, 0, 0))), t_end=0.05)
    _same(pb)


@pytest.mark.parametrize("kind", ["pass", "slab", "shell"])
def test_momentum_boundaries_at_a_shock(kind):
    p_b = 0.995  # momenta fall through it in this set-up (expansion where the particles start)
    bnd = {"pass": (BoundaryMomentumPass(), B(DC(), -1, [0]).double(p_b)),
           "slab": (BoundaryMomentumInjectRestrictSlab(), B(DC(), 1, [0]).double(p_b).vec((-0.5, 0, 0)).vec((0.5, 0, 0))
                    .vec((1.0, 0, 0))),
           "shell": (BoundaryMomentumInjectRestrictShell(), B(DC(), 1, [0]).double(p_b).vec((0, 0, 0)).double(0.01)
                     .double(0.5))}[kind]
    c = distro_header(DC(), (20, 0, 0), (0.9, 0, 0), (1.2, 0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    pb = _parker(bg=_shock(), bnds=[bnd], dist=dist, diff=(DiffusionFullConstant(), DC().double(0.01).double(0.01)),
                 t_end=0.5)
    _same(pb)


def test_sharp_shock_background():
    _same(_parker(bg=_shock(smooth=False), t_end=0.1))


# -- initial conditions ----------------------------------------------------------------------------
INITIAL_CASES = {
    "time_interval": {"it": (InitialTimeInterval(), DC().double(0.0).double(0.05).int(0))},
    "space_line": {"is_": (InitialSpaceLine(), DC().vec((-0.2, 0, 0)).vec((0.2, 0.1, 0)).int(0))},
    "space_box": {"is_": (InitialSpaceBox(), DC().vec((-0.2, -0.2, -0.2)).vec((0.2, 0.2, 0.2)).int(0))},
    "space_circle": {"is_": (InitialSpaceCircle(), DC().vec((0, 0, 0)).vec((0, 0.6, 0.8)).double(0.3))},
    "space_sphere": {"is_": (InitialSpaceSphere(), DC().vec((0.1, 0, 0)).double(0.3))},
    "space_sector": {"is_": (InitialSpaceSphereSector(), DC().vec((0, 0, 0)).double(0.3).double(0.5).double(1.2)
                             .double(0.3).double(2.0))},
    "space_rankine": {"is_": (InitialSpaceRankineHalfBody(), DC().vec((0, 0, 0)).double(0.2).double(0.5))},
    "space_cylinder": {"is_": (InitialSpaceCylinder(), DC().vec((0.1, 0, 0)).vec((0, 0.2, 0.3)).vec((0.3, 0, 0)))},
    "space_cylinder_sector": {"is_": (InitialSpaceCylinderSector(), DC().vec((0.1, 0, 0)).vec((0, 0.2, 0.3))
                                      .vec((0.3, 0, 0)).double(0.5).double(2.5))},
    "momentum_thick_shell_lin": {"im": (InitialMomentumThickShell(), DC().double(0.5).double(2.0).bool(False))},
    "momentum_thick_shell_log": {"im": (InitialMomentumThickShell(), DC().double(0.5).double(2.0).bool(True))},
    "momentum_maxwell": {"im": (InitialMomentumMaxwell(), DC().double(1.0).double(0.3).double(0.2))},
}


@pytest.mark.parametrize("name", sorted(INITIAL_CASES))
def test_initial_classes(name):
    c = distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (3.0, 0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(0).int(0))
    _same(_parker(dist=dist, t_end=0.05, **INITIAL_CASES[name]))


@pytest.mark.parametrize("name", ["beam", "ring", "maxwell", "shell"])
def test_focused_momentum_initials(name):
    """The momentum samplers in the focused (p, mu) coordinates, recorded in (p, mu)."""
    im = {"beam": (InitialMomentumBeam(), DC().double(1.0)),
          "ring": (InitialMomentumRing(), DC().double(1.0).double(0.7)),
          "maxwell": (InitialMomentumMaxwell(), DC().double(1.0).double(0.3).double(0.2)),
          "shell": (InitialMomentumShell(), DC().double(1.0))}[name]
    c = distro_header(DC(), (10, 10, 0), (0.0, -1.0, 0), (3.0, 1.0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(0).int(0))
    _same(_parker(traj=TRAJ_FOCUSED, im=im, dist=dist, diff=False, t_end=0.05))


@pytest.mark.parametrize("name", ["fixed", "beam", "ring", "maxwell"])
def test_lorentz_momentum_initials(name):
    """The samplers in Cartesian momentum about the local field (Lorentz)."""
    im = {"fixed": (InitialMomentumFixed(), DC().vec((0.3, 0.4, 0.5))),
          "beam": (InitialMomentumBeam(), DC().double(1.0)),
          "ring": (InitialMomentumRing(), DC().double(1.0).double(0.7)),
          "maxwell": (InitialMomentumMaxwell(), DC().double(1.0).double(0.3).double(0.2))}[name]
    c = distro_header(DC(), (10, 10, 0), (0.0, -1.0, 0), (3.0, 1.0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(0).int(1))
    pb = _parker(traj=TRAJ_LORENTZ, im=im, dist=dist, diff=False, t_end=0.01)
    pb.options[W.SPX_OPT_STEPS_PER_ORBIT] = 100.0
    _same(pb)


# -- diffusion models ------------------------------------------------------------------------------
def _sw_bg():
    return BackgroundSolarWind(), W.solarwind_params(DC())


_R1 = U.Rigidity(U.mev_to_mom(1000.0))  # 1 GV-ish reference rigidity
_B5 = 5.0e-5 / U.unit_magnetic          # 5 nT
_LAM = 0.1 * W.ONE_AU

DIFFUSION_CASES = {
    "para_constant": ((DiffusionParaConstant(), DC().double(1.0)), None),
    "flow_momentum": ((DiffusionFlowMomentumPowerLaw(), DC().double(0.5).double(0.5).double(0.3).double(1.0).double(0.5)
                       .double(0.1)), "flow"),
    # kap0, T0, r0, pow_law_T, pow_law_r, kap_rat, stream_dep_idx, u_up, w_sh, s_sh
    "kin_energy_radial": ((DiffusionKineticEnergyRadialDistancePowerLaw(),
                           DC().double(0.5).double(1.0).double(0.2).double(0.5).double(1.0).double(0.1).int(0).double(1.0)
                           .double(0.1).double(4.0)), "offset"),
    # LISM_idx, lam_in, lam_out, R0, B0, kap_rat_in, kap_rat_out
    "strauss": ((DiffusionStraussEtAl2013(), DC().int(-1).double(_LAM).double(_LAM).double(_R1).double(_B5).double(0.02)
                 .double(0.02)), "sw"),
    # LISM_idx, kappa_in, kappa_out, R0, B0, kap_rat_in, kap_rat_out
    "potgieter": ((DiffusionPotgieterEtAl2015(), DC().int(-1).double(500.0).double(500.0).double(_R1).double(_B5)
                   .double(0.02).double(0.02)), "sw"),
    # lam_para, lam_perp, R0, B0, Bmix_idx, kap_rat_red, radial_limit_perp_red, solar_cycle_idx, solar_cycle_effect
    "empirical": ((DiffusionEmpiricalSOQLTandUNLT(), DC().double(_LAM).double(0.01 * _LAM).double(_R1).double(_B5)
                   .int(0).double(0.5).double(50.0 * W.ONE_AU).int(0).double(0.5)), "sw"),
}


@pytest.mark.parametrize("name", sorted(DIFFUSION_CASES))
def test_diffusion_models(name):
    diff, where = DIFFUSION_CASES[name]
    if where == "sw":
        au = W.ONE_AU
        c = distro_header(DC(), (20, 0, 0), (0.5 * au, 0, 0), (1.5 * au, 0, 0))
        dist = (DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(1))
        pb = _parker(bg=_sw_bg(), diff=diff, is_=(InitialSpaceFixed(), DC().vec((au, 0, 0))),
                     im=(InitialMomentumShell(), DC().double(U.mev_to_mom(100.0))), dist=dist, t_end=0.002, n=12)
    elif where == "offset":
        pb = _parker(diff=diff, is_=(InitialSpaceFixed(), DC().vec((0.3, 0, 0))))
    elif where == "flow":
        bg = (BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0.5, 0, 0)).vec((0, 0, 1.0)).double(0.05))
        pb = _parker(bg=bg, diff=diff)
    else:
        pb = _parker(diff=diff)
    _same(pb)


def test_qlt_pitch_angle_diffusion():
    """DiffusionQLTConstant (D_mumu) in the guiding-centre scattering type."""
    c = distro_header(DC(), (0, 20, 0), (0.0, -1.0, 0), (1.0, 1.0, 1.0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(1))
    pb = _parker(traj=TRAJ_GUIDING_SCATT, diff=(DiffusionQLTConstant(), DC().double(0.1).double(1.0).double(5.0 / 3.0)),
                 dist=dist, t_end=0.5, im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))), n=12)
    _same(pb)


# -- distributions -------------------------------------------------------------------------------
DIST_CASES = {
    "cumulative1": (DistributionPositionCumulativeOrder1(), distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (0.2, 0, 0),
                                                                         width=3)),
    "cumulative2": (DistributionPositionCumulativeOrder2(), distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (0.2, 0, 0),
                                                                         width=9)),
    "position_momentum": (DistributionPositionMomentumUniform(),
                          distro_header(DC(), (10, 10, 0), (-1.0, 0.5, 0), (1.0, 1.5, 0)).double(1.0).double(0.0).int(1)
                          .int(3).int(0)),
}


@pytest.mark.parametrize("name", sorted(DIST_CASES))
def test_distribution_classes(name):
    _same(_parker(dist=DIST_CASES[name]))


def test_divergence_flow_distribution_at_a_shock():
    c = distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (2.0, 0, 0))
    dist = (DistributionDivergenceFlowPowerLaw(), c.double(2.0).double(1.5).double(0.0))
    _same(_parker(bg=_shock(), dist=dist, t_end=0.05))


def test_bent_power_law_spectrum():
    """The modulation set-up with its spectrum recorded by the bent power law (T_b = 1 GeV)."""
    from spectrum_gb300.datacontainer import read_records
    from spectrum_gb300.problem import PluginEntry
    pb = W.gcr_modulation(n_traj=6, energies_mev=[3000.0], t_max_years=0.05)[0]
    for i, e in enumerate(pb.plugins):
        if type(e.plugin).__name__ == "DistributionSpectrumKineticEnergyPowerLaw":
            c = DC()
            for rec in read_records(e.blob):  # the power-law container, then T_b, pow_law_b, bend
                c._add(rec)
            c.double(1000.0 * U.MEV / U.unit_energy).double(1.5).double(2.0)
            pb.plugins[i] = PluginEntry(DistributionSpectrumKineticEnergyBentPowerLaw(), c.data(), c.size())
    _same(pb)


# -- the Parker source type ---------------------------------------------------------------------------
def test_parker_source_injection():
    """TrajectoryParkerSource with SourceMomentumInjection (backward in time at a smooth shock)."""
    src = (SourceMomentumInjection(), DC().double(1.0).double(2.0))
    c = distro_header(DC(), (10, 0, 0), (0.5, 0, 0), (2.0, 0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    pb = _parker(traj=TRAJ_PARKER_SOURCE, flow=BACKWARD, bg=_shock(), src=src, dist=dist,
                 im=(InitialMomentumShell(), DC().double(0.95)), t_end=-0.2, n=16)
    r = _same(pb)
    assert (r.traj["amp"] != 0.0).sum() >= 4  # momenta rise through p_inj = 1 and the source injects


def test_parker_source_constant():
    """TrajectoryParkerSource with SourceConstant: the amplitude grows by S0 dt exp(weight) every step."""
    src = (SourceConstant(), DC().double(0.7))
    pb = _parker(traj=TRAJ_PARKER_SOURCE, flow=BACKWARD, src=src, t_end=-0.05, n=12)
    r = _same(pb)
    # the time boundary ends the run a few 1e-8 past |t| = 0.05, as the reference's proximity check does
    np.testing.assert_allclose(r.traj["amp"], 0.7 * np.abs(r.traj["t"]), rtol=1e-12)


def _spherical_source_problem():
    src = (SourceSphericalShockInjection(), DC().double(1.0).vec((0, 0, 0)).double(0.0).double(0.2).double(2.0))
    c = distro_header(DC(), (10, 0, 0), (0.5, 0, 0), (2.0, 0, 0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    return _parker(traj=TRAJ_PARKER_SOURCE, flow=BACKWARD, bg=_shock(), src=src, dist=dist,
                   im=(InitialMomentumShell(), DC().double(0.95)), t_end=-0.2, n=24)


def test_parker_source_spherical_shell_injection():
    """SourceSphericalShockInjection: injection at p_inj only within 0.2 of the origin."""
    r = _same(_spherical_source_problem())
    injected = (r.traj["amp"] != 0.0).sum()
    assert 0 < injected < len(r.traj), injected  # both sides of the shell condition


# -- backward time for the Runge-Kutta types, forward time for the source type --------------------------
def _lorentz_backward():
    # the reference's compiled steps per orbit (src/trajectory_lorentz.hh:26), which its harness runs with
    pb = _parker(traj=TRAJ_LORENTZ, flow=BACKWARD, diff=False, t_end=-0.1, n=12)
    pb.options[W.SPX_OPT_STEPS_PER_ORBIT] = 100.0
    return pb


def _focused_backward():
    au = W.ONE_AU
    c = distro_header(DC(), (20, 0, 0), (0.5 * au, 0, 0), (1.5 * au, 0, 0))
    dist = (DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(1))
    return _parker(traj=TRAJ_FOCUSED, flow=BACKWARD, diff=False, bg=_sw_bg(), dist=dist, n=12, t_end=-2000.0,
                   is_=(InitialSpaceFixed(), DC().vec((au, 0, 0))),
                   im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))))


def _guiding_diff_scatt_backward():
    return _parker(traj=TRAJ_GUIDING_DIFF_SCATT, flow=BACKWARD, diff=(DiffusionPerpConstant(), DC().double(0.05)),
                   im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))), t_end=-0.5, n=12)


def _parker_source_forward():
    return _parker(traj=TRAJ_PARKER_SOURCE, flow=FORWARD, src=(SourceConstant(), DC().double(0.3)), t_end=0.05, n=12)


TIME_FLOW_CASES = {"lorentz_backward": _lorentz_backward, "focused_backward": _focused_backward,
                   "guiding_diff_scatt_backward": _guiding_diff_scatt_backward,
                   "parker_source_forward": _parker_source_forward}


@pytest.mark.parametrize("name", sorted(TIME_FLOW_CASES))
def test_time_flow_variants(name):
    r = _same(TIME_FLOW_CASES[name]())
    assert (r.traj["steps"] > 1).all()


# -- more background and trajectory combinations --------------------------------------------------------
def _dipole_bg():
    from spectrum_gb300.plugins import BackgroundDipole
    r_e = W.R_EARTH_CM / U.unit_length
    b_eq = W.B_EARTH_G / U.unit_magnetic
    c = DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
    return (BackgroundDipole(), c.double(r_e).double(0.1)), r_e


def _moving_smooth_shock():
    """A smooth shock moving at 0.5 with an oblique field: dU/dt and grad U both nonzero."""
    c = DC().double(0.0).vec((0, 0, 0)).vec((1.0, 0, 0)).vec((0.3, 0.2, 1.0)).double(0.02)
    c.vec((1.0, 0, 0)).double(0.5).double(4.0)
    return BackgroundSmoothShock(), c.double(0.05).double(0.1)


def _combo(name):
    if name == "parker_dipole":
        bg, r_e = _dipole_bg()
        return _parker(bg=bg, diff=(DiffusionFullConstant(), DC().double(1e-4).double(1e-3)), t_end=1.0, n=12,
                       is_=(InitialSpaceFixed(), DC().vec((3.0 * r_e, 0, 0.1 * r_e))))
    if name == "parker_backward_smooth_shock":
        return _parker(bg=_shock(), flow=BACKWARD, diff=(DiffusionFullConstant(), DC().double(0.01).double(0.01)),
                       t_end=-0.5, n=12)
    if name == "focused_moving_smooth_shock":
        return _parker(traj=TRAJ_FOCUSED, bg=_moving_smooth_shock(), diff=False, t_end=0.3, n=12,
                       is_=(InitialSpaceFixed(), DC().vec((-0.2, 0, 0))))
    if name == "lorentz_sharp_shock":
        pb = _parker(traj=TRAJ_LORENTZ, bg=_shock(smooth=False), diff=False, t_end=0.3, n=12,
                     is_=(InitialSpaceFixed(), DC().vec((-0.05, 0, 0))))
        pb.options[W.SPX_OPT_STEPS_PER_ORBIT] = 100.0
        return pb
    raise KeyError(name)


COMBO_CASES = ["focused_moving_smooth_shock", "lorentz_sharp_shock", "parker_backward_smooth_shock", "parker_dipole"]


@pytest.mark.parametrize("name", COMBO_CASES)
def test_background_trajectory_combinations(name):
    r = _same(_combo(name))
    assert (r.traj["steps"] > 1).all()


# -- the weakly nonlinear models: K_perp with the QLT pitch-angle coefficient ---------------------------------
def _wnlt(ramp=False):
    """A2A 0.1, l_max 1, ps_index 5/3, A2T = A2L = 0.1; the ramp from l_max_HP 0.3 at z_nose 0.1 to the
    sheath at 0.6, which the trajectories starting at (0.3, 0, 0.2) (z0 = 0.32) cross both ways."""
    c = DC().double(0.1).double(1.0).double(5.0 / 3.0).double(0.1).double(0.1)
    if ramp:
        return DiffusionWNLTRampVLISM(), c.double(0.3).double(0.1).double(0.6)
    return DiffusionWNLTConstant(), c


def _wnlt_problem(traj, ramp, mu_method=0, dipole=False, t_end=0.3):
    c = distro_header(DC(), (0, 20, 0), (0.0, -1.0, 0), (1.0, 1.0, 1.0))
    dist = (DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(1))
    kw = {}
    if dipole:
        kw["bg"] = (BackgroundDipole(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, -1.0)).double(0.05)
                    .double(1.0).double(0.1))
    pb = _parker(traj=traj, diff=_wnlt(ramp), dist=dist, t_end=t_end, n=12,
                 is_=(InitialSpaceFixed(), DC().vec((1.5, 0, 0.2) if dipole else (0.3, 0, 0.2))),
                 im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))), **kw)
    if mu_method:
        pb.options[W.SPX_OPT_MU_METHOD] = float(mu_method)
    return pb


WNLT_CASES = {
    "constant_guiding_diff_scatt": lambda: _wnlt_problem(TRAJ_GUIDING_DIFF_SCATT, False),
    "constant_guiding_diff_scatt_dipole": lambda: _wnlt_problem(TRAJ_GUIDING_DIFF_SCATT, False, dipole=True),
    "ramp_guiding_diff_scatt": lambda: _wnlt_problem(TRAJ_GUIDING_DIFF_SCATT, True),
    "ramp_guiding_diff": lambda: _wnlt_problem(TRAJ_GUIDING_DIFF, True),
    "ramp_guiding_scatt": lambda: _wnlt_problem(TRAJ_GUIDING_SCATT, True, t_end=1.0),
    "ramp_guiding_scatt_milstein": lambda: _wnlt_problem(TRAJ_GUIDING_SCATT, True, mu_method=1, t_end=1.0),
    "ramp_guiding_scatt_rk2": lambda: _wnlt_problem(TRAJ_GUIDING_SCATT, True, mu_method=2, t_end=1.0),
}


@pytest.mark.parametrize("name", sorted(WNLT_CASES))
def test_wnlt_diffusion(name):
    r = _same(WNLT_CASES[name]())
    assert (r.traj["steps"] > 3).all()


# -- the perpendicular Milstein and RK2 schemes (STOCHASTIC_METHOD_PERP 1, 2) --------------------------------------
# The reference evaluates the displaced points into a SpatialData whose field mask is never initialised
# (src/trajectory_guiding_diff.cc:133, 188), so which fields reach the diffusion model there is undefined. The
# cases are chosen so that nothing depends on it: a uniform |B|, with D_perp varying through the position alone
# (the WNLT ramp) or constant.
def _perp_problem(traj, perp_method, ramp=True):
    pb = _wnlt_problem(traj, True) if ramp else _parker(
        traj=traj, diff=(DiffusionPerpConstant(), DC().double(0.05)), t_end=0.3, n=12,
        im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))))
    pb.options[W.SPX_OPT_PERP_METHOD] = float(perp_method)
    return pb


PERP_CASES = {
    "milstein_ramp_guiding_diff": lambda: _perp_problem(TRAJ_GUIDING_DIFF, 1),
    "rk2_ramp_guiding_diff": lambda: _perp_problem(TRAJ_GUIDING_DIFF, 2),
    "milstein_constant_guiding_diff": lambda: _perp_problem(TRAJ_GUIDING_DIFF, 1, ramp=False),
    "rk2_constant_guiding_diff": lambda: _perp_problem(TRAJ_GUIDING_DIFF, 2, ramp=False),
    "rk2_ramp_guiding_diff_scatt": lambda: _perp_problem(TRAJ_GUIDING_DIFF_SCATT, 2),
    "rk2_ramp_guiding_diff_absorbed": lambda: _perp_absorbed(),
}


def _perp_absorbed():
    """RK2 with an absorbing sphere that the trajectories reach: a trial point of the scheme can cross it
    (src/trajectory_guiding_diff.cc:205, 214), which ends the trajectory there."""
    pb = _perp_problem(TRAJ_GUIDING_DIFF, 2)
    pb.AddBoundary(BoundarySphereAbsorb(), B(DC(), 1, [0]).vec((0.3, 0, 0.2)).double(0.25))
    return pb


@pytest.mark.parametrize("name", sorted(PERP_CASES))
def test_perpendicular_schemes(name):
    r = _same(PERP_CASES[name]())
    assert (r.traj["steps"] > 3).all()


# -- DistributionLossCone (src/distribution_other.cc:794-862) ------------------------------------------
# The |B| extrema it reads are tracked by the reference only when compiled with RECORD_BMAG_EXTREMA
# (src/trajectory_base.hh:31); the reference harness variants *_bmag are built that way. Orbits in the
# dipole: |B| changes by a factor of several along a bounce.
def _losscone_problem(traj, val_time=1, val_coord=0, n=6):
    import math
    from spectrum_gb300.plugins import DistributionLossCone
    r_e = W.R_EARTH_CM / U.unit_length
    b_eq = W.B_EARTH_G / U.unit_magnetic
    bg = (BackgroundDipole(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
          .double(r_e).double(0.1))
    if val_coord == 1:
        lo, hi = (2.0 * r_e, 0.0, 0.0), (6.0 * r_e, math.pi, 2.0 * math.pi)
    else:
        lo, hi = (-6.0 * r_e,) * 3, (6.0 * r_e,) * 3
    c = distro_header(DC(), (6, 6, 6), lo, hi, bin_outside=(1, 1, 1), width=3)
    dist = (DistributionLossCone(), c.int(val_time).int(val_coord))
    kw = dict(diff=(DiffusionFullConstant(), DC().double(1e-4).double(1e-3)), t_end=1.0) if traj == TRAJ_PARKER else \
        dict(diff=False, t_end=(10.0 if traj == TRAJ_GUIDING else 0.3) / U.unit_time)
    return _parker(traj=traj, bg=bg, dist=dist, n=n, is_=(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0))),
                   im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))), **kw)


LOSSCONE_CASES = {
    "guiding_final_cartesian": lambda: _losscone_problem(TRAJ_GUIDING),
    "guiding_initial_spherical": lambda: _losscone_problem(TRAJ_GUIDING, val_time=0, val_coord=1),
    "lorentz_final_spherical": lambda: _losscone_problem(TRAJ_LORENTZ, val_coord=1),
    "parker_final_cartesian": lambda: _losscone_problem(TRAJ_PARKER),
}


# -- DistributionAnisotropyLISM (src/distribution_other.cc:364-483, Lorentz only) ----------------------
# Dipole orbits from a fixed point; each case sends the time boundary's event to one of the five
# weights. The reference's set-up accepts bins in the first and third dimensions only (dims 5) and
# leaves the third value unset: the third axis has one bin over [-1e300, 1e300] with outliers kept,
# so any finite value lands in it.
def _aniso_problem(action, n=8):
    import math
    from spectrum_gb300.plugins import DistributionAnisotropyLISM
    r_e = W.R_EARTH_CM / U.unit_length
    b_eq = W.B_EARTH_G / U.unit_magnetic
    bg = (BackgroundDipole(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
          .double(r_e).double(0.1))
    c = distro_header(DC(), (9, 0, 1), (0.0, 0.0, -1e300), (math.pi, 1.0, 1e300), bin_outside=(1, 1, 1))
    c3 = 1.0 / math.sqrt(3.0)
    rot = ((c3, c3, c3), (1.0 / math.sqrt(2.0), -1.0 / math.sqrt(2.0), 0.0), (c3 / math.sqrt(2.0), c3 / math.sqrt(2.0), -2.0 * c3 / math.sqrt(2.0)))
    c.vec(rot[0]).vec(rot[1]).vec(rot[2]).vec((2.0e-3, -1.0e-3, 5.0e-4)).double(2.7).vec((0.3, -0.2, 0.1))
    return _parker(traj=TRAJ_LORENTZ, bg=bg, dist=(DistributionAnisotropyLISM(), c), n=n, diff=False,
                   t_end=0.2 / U.unit_time, t_action=(action,),
                   is_=(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0))),
                   im=(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0))))


ANISO_CASES = {f"action{a}": (lambda a=a: _aniso_problem(a)) for a in range(5)}


@pytest.mark.parametrize("name", sorted(ANISO_CASES))
def test_anisotropy_lism(name):
    pb = ANISO_CASES[name]()
    r = _same(pb)
    counts, sums, n_ev = r.distros[0]
    assert n_ev == len(r.traj) and counts.sum() == len(r.traj)
    assert np.isfinite(sums).all() and (sums != 0.0).any()


def test_anisotropy_lism_refused_outside_lorentz():
    """The class exists for Lorentz trajectories only; dims other than 5 fail its set-up."""
    from spectrum_gb300.plugins import DistributionAnisotropyLISM
    pb = _aniso_problem(0)
    pb.traj = TRAJ_GUIDING
    with pytest.raises(Exception):
        ot.run_oracle(pb)
    c = distro_header(DC(), (9, 4, 0), (0.0, 0.0, 0.0), (3.0, 6.0, 1.0))
    c.vec((1, 0, 0)).vec((0, 1, 0)).vec((0, 0, 1)).vec((0, 0, 0)).double(2.7).vec((0, 0, 0))
    pb = _aniso_problem(0)
    pb.plugins[-1] = type(pb.plugins[-1])(DistributionAnisotropyLISM(), c.data(), c.size())
    with pytest.raises(Exception):
        ot.run_oracle(pb)


@pytest.mark.parametrize("name", sorted(LOSSCONE_CASES))
def test_loss_cone(name):
    pb = LOSSCONE_CASES[name]()
    if ot.ref_binary(pb) is None:
        pytest.skip("reference harness with RECORD_BMAG_EXTREMA not built (needs the reference sources)")
    r = _same(pb)
    counts, sums, n_ev = r.distros[0]
    assert n_ev == len(r.traj)
    # the extrema bracket the field at the start, and the half-angle lies in (0, pi/2]. A Runge-Kutta
    # event reads |B| at the step's last stage point, which can exceed the maximum along the stored
    # points: the reference's asin then gives NaN, which both sides carry alike.
    bmin, bmax, ang = (sums[counts > 0] / counts[counts > 0][:, None]).T
    ok = np.isfinite(ang)
    assert (bmin < bmax).all() and (ang[ok] > 0).all() and (ang[ok] <= np.pi / 2 + 1e-12).all()
    assert ok.any()


# -- TrajectoryFieldline (src/trajectory_fieldline.cc): the field-line tracer ----------------------------
# Lines of the dipole traced from random points of a sphere of 3 Earth radii at the parallel speed of the
# momentum's third component; the fields are B only (which_field_to_follow), the step 0.5 dmax / |v_para|.
# The outer sphere absorbs the lines that reach 8 radii, the inner one reflects (ReverseMomentum negates the
# whole momentum), and the final points are binned in spherical coordinates.
def _fieldline_problem(flow=FORWARD, rk=25, im=None, dist=None, reflect=True, n=8, t_end=None, bg=None, scale=None):
    r_e = scale or W.R_EARTH_CM / U.unit_length  # the length scale of the set-up
    b_eq = W.B_EARTH_G / U.unit_magnetic
    if bg is None:
        bg = (BackgroundDipole(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq))
              .double(0.2 * r_e).double(r_e).double(0.05))
    if dist is None:
        import math
        c = distro_header(DC(), (8, 8, 8), (0.5 * r_e, 0.0, 0.0), (10.0 * r_e, math.pi, 2.0 * math.pi),
                          bin_outside=(1, 1, 1))
        dist = (DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(1))
    p = U.mev_to_mom(1.0)
    if t_end is None:  # long enough to reach the outer sphere
        t_end = (12.0 * r_e / U.Vel(p)) * (1.0 if flow == FORWARD else -1.0)
    pb = _parker(traj=TRAJ_FIELDLINE, flow=flow, bg=bg, diff=False, dist=dist, n=n, t_end=t_end,
                 is_=(InitialSpaceSphere(), DC().vec((0.0, 0.0, 0.0)).double(3.0 * r_e)),
                 im=im or (InitialMomentumShell(), DC().double(p)),
                 bnds=[(BoundarySphereAbsorb(), B(DC(), 1, [0]).vec((0, 0, 0)).double(8.0 * r_e))] +
                      ([(BoundarySphereReflect(), B(DC(), -1, [-1]).vec((0, 0, 0)).double(1.5 * r_e))] if reflect else []))
    pb.rk = rk
    return pb



def _fieldline_spectrum():
    c = distro_header(DC(), (10, 0, 0), (1e-3, 0, 0), (10.0, 0, 0), log_bins=(1, 0, 0), bin_outside=(1, 0, 0))
    # DistributionSpectrumKineticEnergyPowerLaw: J0, T0, power law, cold value
    from spectrum_gb300.plugins import DistributionSpectrumKineticEnergyPowerLaw
    c.double(1.0).double(U.MEV / U.unit_energy).double(-2.5).double(0.0)
    return DistributionSpectrumKineticEnergyPowerLaw(), c


FIELDLINE_CASES = {
    "dipole_rk4": lambda: _fieldline_problem(),
    "dipole_rk4_backward": lambda: _fieldline_problem(flow=BACKWARD),
    "dipole_euler": lambda: _fieldline_problem(rk=0),
    "dipole_dormand_prince": lambda: _fieldline_problem(rk=29),
    # against the field: a fixed momentum with a negative parallel component
    "fixed_antiparallel": lambda: _fieldline_problem(im=(InitialMomentumFixed(), DC().vec((0.3, -0.2, -0.45)))),
    # one uniform per sample (drawn twice at the start, as SetStart samples twice), log-uniform
    "thick_shell_log": lambda: _fieldline_problem(im=(InitialMomentumThickShell(), DC().double(0.2).double(0.9)
                                                      .bool(True))),
    # the mean momentum only, no draws
    "maxwell": lambda: _fieldline_problem(im=(InitialMomentumMaxwell(), DC().double(0.5).double(0.1).double(0.05))),
    # the momentum recorded as (p_para, 0, 0)
    "momentum_spherical": lambda: _fieldline_problem(
        dist=(DistributionMomentumUniform(),
              distro_header(DC(), (10, 0, 0), (-0.5, 0, 0), (0.5, 0, 0)).double(1.0).double(0.0).int(1).int(1)),
        im=(InitialMomentumFixed(), DC().vec((0.0, 0.0, -0.45)))),
    # the parallel component's kinetic energy, with the hot weight of the final (reflected, negative) momentum
    "spectrum": lambda: _fieldline_problem(dist=_fieldline_spectrum()),
    # Parker-spiral lines from 3 au, absorbed at 8 au
    "solar_wind_spiral": lambda: _fieldline_problem(bg=_sw_bg(), reflect=False, n=6, scale=W.ONE_AU),
}


@pytest.mark.parametrize("name", sorted(FIELDLINE_CASES))
def test_fieldline(name):
    pb = FIELDLINE_CASES[name]()
    if ot.ref_binary(pb) is None:
        pytest.skip("reference harness for TrajectoryFieldline not built (needs the reference sources)")
    r = _same(pb)
    assert (r.traj["steps"] > 1).all()


def test_fieldline_refuses_what_the_reference_does_not_have():
    """No momentum boundaries, beam or ring initials, or divergence-flow distribution for field lines."""
    for extra in ("mom_bnd", "beam", "divflow"):
        pb = _fieldline_problem()
        if extra == "mom_bnd":
            pb.AddBoundary(BoundaryMomentumPass(), B(DC(), -1, [0]).double(0.5))
        elif extra == "beam":
            pb.replace(4, 2, InitialMomentumBeam(), DC().double(0.02))
        else:
            pb.AddDistribution(DistributionDivergenceFlowPowerLaw(), distro_header(DC(), (4, 0, 0), (0, 0, 0), (1, 0, 0))
                               .double(1.0).double(1.0).double(0.0))
        with pytest.raises(Exception):
            ot.run_oracle(pb)


# -- BackgroundDiscontinuity and BackgroundSmoothDiscontinuity (src/background_discontinuity.cc,
# src/background_smooth_discontinuity.cc): a moving plane across which U and B jump to a given state, sharp
# or through a tanh of steepness 4 (the smooth shock's is 8). The reference's smooth discontinuity is
# compiled through oracle/ref_glue/smooth_discont_wrap.cc (it names c_code unqualified).
def _discontinuity(smooth):
    from spectrum_gb300.plugins import BackgroundDiscontinuity, BackgroundSmoothDiscontinuity
    c = DC().double(0.0).vec((0, 0, 0)).vec((0.8, 0.1, 0.0)).vec((0.2, 0.1, 1.0)).double(0.02)
    c.vec((1.0, 0.3, 0.0)).double(0.3).vec((0.25, -0.2, 0.05)).vec((0.5, 0.6, 1.4))
    if smooth:
        return BackgroundSmoothDiscontinuity(), c.double(0.05).double(0.1)
    return BackgroundDiscontinuity(), c


def _discontinuity_problem(traj, smooth, flow=FORWARD, n=12):
    c = distro_header(DC(), (20, 0, 0), (-1.0, 0, 0), (1.0, 0, 0), bin_outside=(1, 0, 0))
    dist = (DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(0))
    kw = dict(diff=(DiffusionFullConstant(), DC().double(0.01).double(0.02)), t_end=0.5) if traj == TRAJ_PARKER else \
        dict(diff=False, t_end=0.3)
    pb = _parker(traj=traj, bg=_discontinuity(smooth), dist=dist, n=n, flow=flow,
                 is_=(InitialSpaceFixed(), DC().vec((-0.05, 0.0, 0.0))), **kw)
    if traj == TRAJ_LORENTZ:
        pb.options[W.SPX_OPT_STEPS_PER_ORBIT] = 100.0
    if traj == TRAJ_FIELDLINE:
        pb.replace(4, 2, InitialMomentumShell(), DC().double(0.2))
    return pb


DISCONT_CASES = {
    "parker_sharp": lambda: _discontinuity_problem(TRAJ_PARKER, False),
    "parker_smooth": lambda: _discontinuity_problem(TRAJ_PARKER, True),
    "focused_smooth": lambda: _discontinuity_problem(TRAJ_FOCUSED, True),
    "lorentz_sharp": lambda: _discontinuity_problem(TRAJ_LORENTZ, False),
    "lorentz_smooth": lambda: _discontinuity_problem(TRAJ_LORENTZ, True),
    "fieldline_smooth": lambda: _discontinuity_problem(TRAJ_FIELDLINE, True),
}


@pytest.mark.parametrize("name", sorted(DISCONT_CASES))
def test_discontinuity_backgrounds(name):
    pb = DISCONT_CASES[name]()
    if ot.ref_binary(pb) is None:
        pytest.skip("reference harness not built for this trajectory type")
    r = _same(pb)
    assert (r.traj["steps"] > 1).all()
