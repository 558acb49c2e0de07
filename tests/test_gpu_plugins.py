"""Every plugin class on the device: the FP64 kernel against the oracle, trajectory by trajectory,
on the one-class-at-a-time problems whose oracle runs tests/test_oracle_plugins.py pins bit for
bit to the reference's own code. Every trajectory takes the same steps to the same outcome, every
histogram bin and event count is equal, and positions agree to within a fixed multiple of the
spread the oracle itself shows when its normal deviates change by one ulp
(oracle_tools.assert_fp64_parity): the device's log, sin and cos may round the last bit
differently from the host's, and some schemes amplify that (the perpendicular RK2 scheme's second
differences over 1e-4 dmax by about 1e8 a step)."""
import numpy as np
import pytest

import oracle_tools as ot
import test_oracle_plugins as cases
from spectrum_gb300 import capi
from spectrum_gb300.datacontainer import DataContainer as DC
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu


def _problems():
    out = {}
    for k, v in cases.BOUNDARY_CASES.items():
        out["boundary_" + k] = lambda v=v: cases._parker(bnds=[v])
    for k, v in cases.INITIAL_CASES.items():
        def make(v=v):
            c = cases.distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (3.0, 0, 0))
            dist = (cases.DistributionMomentumUniform(), c.double(1.0).double(0.0).int(0).int(0))
            return cases._parker(dist=dist, t_end=0.05, **v)
        out["initial_" + k] = make
    for k in cases.DIST_CASES:
        out["distribution_" + k] = lambda k=k: cases._parker(dist=cases.DIST_CASES[k])
    out["sharp_shock"] = lambda: cases._parker(bg=cases._shock(smooth=False), t_end=0.1)
    out["region_absorb"] = lambda: cases._parker(
        bg=cases._shock(smooth=False), bnds=[(cases.BoundaryRegionAbsorb(), cases.B(DC(), 1, [0]).int(0).double(1.5))],
        is_=(cases.InitialSpaceFixed(), DC().vec((-0.05, 0, 0))), t_end=0.05)
    for k, (diff, where) in cases.DIFFUSION_CASES.items():
        out["diffusion_" + k] = lambda k=k: _diffusion_case(k)
    for kind in ("pass", "slab", "shell"):
        out["momentum_boundary_" + kind] = lambda kind=kind: _momentum_case(kind)
    for name in ("beam", "ring", "maxwell", "shell"):
        out["focused_initial_" + name] = lambda name=name: _focused_initial(name)
    out["divergence_flow"] = lambda: cases._parker(
        bg=cases._shock(), t_end=0.05,
        dist=(cases.DistributionDivergenceFlowPowerLaw(),
              cases.distro_header(DC(), (10, 0, 0), (0.0, 0, 0), (2.0, 0, 0)).double(2.0).double(1.5).double(0.0)))
    out["parker_source"] = _source_case
    out["parker_source_spherical"] = cases._spherical_source_problem
    out["lorentz_solar_wind"] = _lorentz_solar_wind
    for name, make in cases.WNLT_CASES.items():
        out["wnlt_" + name] = make
    for name, make in cases.PERP_CASES.items():
        out["perp_" + name] = make
    for name in cases.COMBO_CASES:
        out["combination_" + name] = lambda name=name: cases._combo(name)
    for name, make in cases.LOSSCONE_CASES.items():
        out["loss_cone_" + name] = make
    for name, make in cases.ANISO_CASES.items():
        out["anisotropy_lism_" + name] = make
    for name, make in cases.DISCONT_CASES.items():
        if not name.startswith("fieldline"):  # the field-line case runs with the other field lines
            out["discontinuity_" + name] = make
    out["parker_source_constant"] = lambda: cases._parker(
        traj=cases.TRAJ_PARKER_SOURCE, flow=cases.BACKWARD, src=(cases.SourceConstant(), DC().double(0.7)),
        t_end=-0.05, n=12)
    return out


def _diffusion_case(name):
    diff, where = cases.DIFFUSION_CASES[name]
    if where == "sw":
        au = cases.W.ONE_AU
        c = cases.distro_header(DC(), (20, 0, 0), (0.5 * au, 0, 0), (1.5 * au, 0, 0))
        dist = (cases.DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(1))
        return cases._parker(bg=cases._sw_bg(), diff=diff, is_=(cases.InitialSpaceFixed(), DC().vec((au, 0, 0))),
                             im=(cases.InitialMomentumShell(), DC().double(cases.U.mev_to_mom(100.0))), dist=dist,
                             t_end=0.002, n=12)
    if where == "offset":
        return cases._parker(diff=diff, is_=(cases.InitialSpaceFixed(), DC().vec((0.3, 0, 0))))
    if where == "flow":
        bg = (cases.BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0.5, 0, 0)).vec((0, 0, 1.0)).double(0.05))
        return cases._parker(bg=bg, diff=diff)
    return cases._parker(diff=diff)


def _momentum_case(kind):
    p_b = 0.995
    B = cases.B
    bnd = {"pass": (cases.BoundaryMomentumPass(), B(DC(), -1, [0]).double(p_b)),
           "slab": (cases.BoundaryMomentumInjectRestrictSlab(), B(DC(), 1, [0]).double(p_b).vec((-0.5, 0, 0))
                    .vec((0.5, 0, 0)).vec((1.0, 0, 0))),
           "shell": (cases.BoundaryMomentumInjectRestrictShell(), B(DC(), 1, [0]).double(p_b).vec((0, 0, 0))
                     .double(0.01).double(0.5))}[kind]
    c = cases.distro_header(DC(), (20, 0, 0), (0.9, 0, 0), (1.2, 0, 0))
    dist = (cases.DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    return cases._parker(bg=cases._shock(), bnds=[bnd], dist=dist,
                         diff=(cases.DiffusionFullConstant(), DC().double(0.01).double(0.01)), t_end=0.5)


def _focused_initial(name):
    im = {"beam": (cases.InitialMomentumBeam(), DC().double(1.0)),
          "ring": (cases.InitialMomentumRing(), DC().double(1.0).double(0.7)),
          "maxwell": (cases.InitialMomentumMaxwell(), DC().double(1.0).double(0.3).double(0.2)),
          "shell": (cases.InitialMomentumShell(), DC().double(1.0))}[name]
    c = cases.distro_header(DC(), (10, 10, 0), (0.0, -1.0, 0), (3.0, 1.0, 0))
    dist = (cases.DistributionMomentumUniform(), c.double(1.0).double(0.0).int(0).int(0))
    return cases._parker(traj=cases.TRAJ_FOCUSED, im=im, dist=dist, diff=False, t_end=0.05)


def _source_case():
    src = (cases.SourceMomentumInjection(), DC().double(1.0).double(2.0))
    c = cases.distro_header(DC(), (10, 0, 0), (0.5, 0, 0), (2.0, 0, 0))
    dist = (cases.DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    return cases._parker(traj=cases.TRAJ_PARKER_SOURCE, flow=cases.BACKWARD, bg=cases._shock(), src=src, dist=dist,
                         im=(cases.InitialMomentumShell(), DC().double(0.95)), t_end=-0.2, n=16)


def _lorentz_solar_wind():
    """Full orbits in the solar wind, where E = -U x B / c (deviation D4: the reference's solar wind leaves U
    unset under the Lorentz mask, so this case is checked against the oracle only)."""
    au = cases.W.ONE_AU
    c = cases.distro_header(DC(), (20, 0, 0), (0.0, 0, 0), (2.0 * au, 0, 0))
    dist = (cases.DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(1))
    return cases._parker(traj=cases.TRAJ_LORENTZ, diff=False, bg=cases._sw_bg(), dist=dist, n=24, t_end=2.0,
                         is_=(cases.InitialSpaceFixed(), DC().vec((au, 0.1 * au, 0.05 * au))),
                         im=(cases.InitialMomentumShell(), DC().double(cases.U.mev_to_mom(10.0))))


PROBLEMS = _problems()


def _check(pb):
    res = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    ot.assert_fp64_parity(res.records[0], ref, ot.run_oracle(pb, nudge_libm=1), distros=res.distros[0])


@pytest.mark.parametrize("name", sorted(PROBLEMS))
def test_plugin_class_on_device(built_lib, name):
    _check(PROBLEMS[name]())
