"""Butcher tables beyond Euler and RK4, and adaptive stepping, in the oracle against the reference's
own code compiled with each table (RK_INTEGRATOR_TYPE; oracle/Makefile variants *_rk<N>).

The reference's RKSlopes (src/trajectory_base.cc:315-357) and RKStep (:366-406): the stages with
the table's lower triangle, the weights v, and for the adaptive tables the lower-order position
with the weights w, the error against 1e-9 (|r| + |r_lo|) + 1e-9, dt_adaptive and the rejection of a
step whose error exceeds 1 (src/trajectory_parker.cc:280-287 for Parker). Each case below is run by
both and compared bit for bit, with deviation D6 reproduced as the reference has it: after a
rejected step the reference keeps the fields of that step's last stage point."""
import os
import sys

import numpy as np
import pytest

import oracle_tools as ot
import test_oracle_plugins as cases
from spectrum_gb300 import workloads as W
from spectrum_gb300.datacontainer import DataContainer as DC
from spectrum_gb300 import units as U
from spectrum_gb300.plugins import BackgroundDipole, DiffusionIsotropicConstant
from spectrum_gb300.problem import BACKWARD, TRAJ_GUIDING, TRAJ_GUIDING_DIFF, TRAJ_GUIDING_SCATT, TRAJ_PARKER_SOURCE

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402

#: the cases in which steps are rejected (the others take the tables' weights without a rejection)
REJECTING = {"lorentz_dipole_rk9", "lorentz_dipole_rk12", "lorentz_dipole_rk13", "lorentz_dipole_rk21",
             "lorentz_dipole_rk32", "focused_solarwind_rk29", "parker_sharp_shock_rk29",
             "guiding_coarse_dipole_rk29", "guidingscatt_coarse_dipole_rk29"}


def _with_rk(pb, rk):
    pb.rk = rk
    return pb


def _parker_source(rk):
    src = (cases.SourceMomentumInjection(), DC().double(1.0).double(2.0))
    c = cases.distro_header(DC(), (10, 0, 0), (0.5, 0, 0), (2.0, 0, 0))
    dist = (cases.DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(0))
    return _with_rk(cases._parker(traj=TRAJ_PARKER_SOURCE, flow=BACKWARD, bg=cases._shock(), src=src, dist=dist,
                                  im=(cases.InitialMomentumShell(), DC().double(0.95)), t_end=-0.2, n=16), rk)


def _coarse_dipole(pb, frac=0.5):
    """The problem's dipole with dmax = frac r (and frac R_E at most): steps long enough for the
    embedded error of the adaptive tables to exceed its tolerance, so steps get rejected."""
    r_e = W.R_EARTH_CM / U.unit_length
    b_eq = W.B_EARTH_G / U.unit_magnetic
    c = DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(frac * r_e).double(r_e).double(frac)
    k = [i for i, e in enumerate(pb.plugins) if isinstance(e.plugin, BackgroundDipole)][0]
    pb.plugins[k] = type(pb.plugins[k])(BackgroundDipole(), c.data(), c.size())
    return pb


def _guiding_scatt_dipole():
    pb = _coarse_dipole(make_golden._guiding_dipole(6))
    pb.traj = TRAJ_GUIDING_SCATT
    pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(0.01))
    return pb


def rk_cases():
    out = {}
    for rk in (3, 9, 12, 13, 16, 21, 26, 27, 28, 29, 31, 32):
        out[f"lorentz_dipole_rk{rk}"] = lambda rk=rk: _with_rk(make_golden._dipole_reference_classes(6), rk)
    out["parker_dipole_rk29"] = lambda: _with_rk(cases._combo("parker_dipole"), 29)
    out["parker_dipole_rk16"] = lambda: _with_rk(cases._combo("parker_dipole"), 16)
    out["parker_solarwind_backward_rk29"] = lambda: _with_rk(
        W.gcr_modulation(n_traj=4, energies_mev=[300.0], t_max_years=0.02)[0], 29)
    out["parker_source_rk29"] = lambda: _parker_source(29)
    out["focused_solarwind_rk29"] = lambda: _with_rk(make_golden._focused_reference_classes(6), 29)
    out["guiding_dipole_rk29"] = lambda: _with_rk(make_golden._guiding_dipole(6), 29)
    out["guidingscatt_slab_rk29"] = lambda: _with_rk(
        make_golden._slab_between_mirrors(TRAJ_GUIDING_SCATT, 8, d0=0.5), 29)
    out["guidingdiff_dipole_rk29"] = lambda: _with_rk(make_golden._guiding_perp(TRAJ_GUIDING_DIFF, 6, dipole=True), 29)
    # cases whose steps the adaptive tables reject
    out["parker_sharp_shock_rk29"] = lambda: _with_rk(cases._parker(
        bg=cases._shock(smooth=False), diff=(cases.DiffusionFullConstant(), DC().double(1e-2).double(1e-2)), t_end=0.1,
        n=12), 29)
    out["guiding_coarse_dipole_rk29"] = lambda: _with_rk(_coarse_dipole(make_golden._guiding_dipole(6)), 29)
    out["guidingscatt_coarse_dipole_rk29"] = lambda: _with_rk(_guiding_scatt_dipole(), 29)
    return out


RK_CASES = rk_cases()


def _needs_ref(pb):
    if ot.ref_binary(pb) is None:
        pytest.skip("reference harness for this table not built (needs the reference sources)")


@pytest.mark.parametrize("name", sorted(RK_CASES))
def test_table_matches_reference(name):
    pb = RK_CASES[name]()
    _needs_ref(pb)
    r = cases._same(pb)
    assert (r.traj["steps"] > 2).all()
    if name in REJECTING:
        ot.run_oracle(pb, reference_quirks=1)
        assert ot.rejections() > 0, "no step was rejected: the rejection path was not exercised"


def test_every_table_runs_in_the_oracle():
    """All 32 tables step the dipole orbits; an unknown table number is refused."""
    for rk in [n for n in range(33) if n != 30]:
        r = ot.run_oracle(_with_rk(make_golden._dipole_reference_classes(2), rk))
        assert (r.traj["steps"] > 0).all(), rk
    with pytest.raises(RuntimeError):
        ot.run_oracle(_with_rk(make_golden._dipole_reference_classes(2), 30))


def test_deviation_d6_after_rejected_steps():
    """Without the quirk the step after a rejection sees the fields of the restored point (D6, what the
    CUDA kernels do); the initial states and outcomes agree, the paths part once a step is rejected."""
    pb = RK_CASES["lorentz_dipole_rk32"]()
    a = ot.run_oracle(pb, reference_quirks=1)
    assert ot.rejections() > 0
    b = ot.run_oracle(pb)
    for f in ("attempts", "t0", "pos0", "mom0"):
        assert np.array_equal(a.traj[f], b.traj[f]), f
    assert not np.array_equal(a.traj["pos"], b.traj["pos"])
