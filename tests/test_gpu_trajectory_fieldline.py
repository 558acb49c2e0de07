"""TrajectoryFieldline on the device: the FP64 kernels against the oracle on the field-line problems
whose oracle runs tests/test_oracle_plugins.py pins bit for bit to the reference's own field-line builds
(dipole lines with a reflecting and an absorbing sphere, both time flows, Euler, RK4 and
Dormand-Prince, the momentum samplers, the momentum and spectrum distributions, Parker-spiral lines,
lines through a moving smooth discontinuity).
Every trajectory takes the same steps to the same outcome, every histogram bin and event count is
equal, and positions agree to within the oracle's own one-ulp libm spread. The FP32 kernels trace the
same dipole lines to within single-precision accuracy."""
import numpy as np
import pytest

import oracle_tools as ot
import test_oracle_plugins as cases
from spectrum_gb300 import capi
from spectrum_gb300.datacontainer import DataContainer as DC
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu


FP64_CASES = {**cases.FIELDLINE_CASES, "smooth_discontinuity": cases.DISCONT_CASES["fieldline_smooth"]}


@pytest.mark.parametrize("name", sorted(FP64_CASES))
def test_fieldline_fp64_equals_the_oracle(built_lib, name):
    pb = FP64_CASES[name]()
    res = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    ot.assert_fp64_parity(res.records[0], ref, ot.run_oracle(pb, nudge_libm=1), distros=res.distros[0])


def test_fieldline_fp32_traces_the_same_lines(built_lib):
    """64 dipole lines in FP32: the same outcome for most lines (a line that grazes the reflecting sphere
    may cross it one step apart), and final points within 1e-3 of the FP64 oracle's where the outcome
    and the step count agree (FP32 fields, float-float positions: a few 1e-6 expected)."""
    pb = cases._fieldline_problem(n=64)
    rec = run_problems(pb, precision=capi.SPX_MIXED, record=True).records[0]
    ref = ot.run_oracle(pb).traj
    same = ((rec["status"] & ot.STATUS_MASK) == (ref["status"] & ot.STATUS_MASK)) & (rec["steps"] == ref["steps"])
    assert same.mean() >= 0.75, same.mean()
    err = ot.rel_pos_err(rec[same], ref[same])
    assert np.median(err) < 1e-3 and err.max() < 1e-2, (np.median(err), err.max())
    # the momentum stays (0, 0, +-p): only its sign changes, at reflections
    assert np.array_equal(np.abs(rec["mom"][:, 2]), np.abs(ref["mom"][:, 2]).astype(np.float32).astype(np.float64)) or \
        np.allclose(np.abs(rec["mom"][:, 2]), np.abs(ref["mom"][:, 2]), rtol=1e-6)


def test_fieldline_refuses_what_the_reference_does_not_have(built_lib):
    """Momentum boundaries, beam and ring initials and the divergence-flow distribution are refused for
    field lines when the plugin is added (SPX_ERR_UNKNOWN_PLUGIN)."""
    pb = cases._fieldline_problem()
    refused = [(cases.BoundaryMomentumPass(), cases.B(DC(), -1, [0]).double(0.5)),
               (cases.InitialMomentumBeam(), DC().double(0.4)),
               (cases.InitialMomentumRing(), DC().double(0.4).double(0.5)),
               (cases.DistributionDivergenceFlowPowerLaw(),
                cases.distro_header(DC(), (4, 0, 0), (0, 0, 0), (1, 0, 0)).double(1.0).double(1.0).double(0.0))]
    for plugin, c in refused:
        ctx = capi.Context(pb.traj, pb.time_flow, pb.rk, capi.SPX_FP64)
        with pytest.raises(capi.SpxError) as e:
            ctx.add_plugin(plugin.role, plugin.kind, c.data(), c.size())
        assert e.value.code == -2
        ctx.close()
