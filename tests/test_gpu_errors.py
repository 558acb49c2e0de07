"""The C ABI's error returns, the counterparts of the reference's set-up exceptions
(common/params.hh:52-90, src/trajectory_base.cc:608-632): each bad set-up is refused with its code,
nothing is launched, and the context stays usable. Needs a device only because contexts do."""
import pytest

from spectrum_gb300 import capi, workloads
from spectrum_gb300.problem import TRAJ_GUIDING_DIFF, TRAJ_PARKER

pytestmark = pytest.mark.gpu


def _ctx_with(pb, skip_role=None, blob_edit=None, kind_edit=None):
    ctx = capi.Context(pb.traj, pb.time_flow, pb.rk, capi.SPX_FP64)
    for e in pb.plugins:
        if e.plugin.role == skip_role:
            continue
        blob, kind = e.blob, e.plugin.kind
        if blob_edit and e.plugin.role == blob_edit[0]:
            blob = blob_edit[1](blob)
        if kind_edit and e.plugin.role == kind_edit[0]:
            kind = kind_edit[1]
        ctx.add_plugin(e.plugin.role, kind, blob, e.n_records)
    return ctx


def _code(fn):
    with pytest.raises(capi.SpxError) as e:
        fn()
    return e.value.code


def test_bad_set_ups_are_refused(built_lib):
    pb = workloads.diffusion_uniform(n_traj=10, t_end=0.01)
    # Butcher table 30 does not compile in the reference; tables other than Euler and RK4 run in FP64 only
    assert _code(lambda: capi.Context(TRAJ_PARKER, 0, 30, capi.SPX_FP64)) == -1
    assert _code(lambda: capi.Context(TRAJ_PARKER, 0, 25, capi.SPX_MIXED)) == -1
    # unknown background class: refused when the plugin is added
    assert _code(lambda: _ctx_with(pb, kind_edit=(0, 99))) == -2
    # the pitch-angle models are not compiled for Parker (src/diffusion_other.hh:17, :126): the QLT and
    # WNLT classes are refused there
    for kind in (2, 12, 13):
        assert _code(lambda: _ctx_with(pb, kind_edit=(1, kind))) == -2
    # parameter blob shorter than the class's list: refused when the plugin is added
    assert _code(lambda: _ctx_with(pb, blob_edit=(0, lambda b: b[: len(b) // 2]))) == -3
    # no time boundary: TrajectoryBase::IsSimmulationReady is false
    ctx = _ctx_with(pb, skip_role=3)
    assert _code(lambda: ctx.add_problem(10, 1)) == -4
    ctx.close()
    # a run before any problem
    ctx = _ctx_with(pb)
    assert _code(lambda: ctx.run()) == -8
    # the context is still usable
    ctx.add_problem(10, 1)
    ctx.run()
    st = ctx.sync()
    assert st.trajectories == 10
    ctx.close()


def test_negative_trajectory_count_is_refused(built_lib):
    pb = workloads.diffusion_uniform(n_traj=10, t_end=0.01)
    ctx = _ctx_with(pb)
    assert _code(lambda: ctx.add_problem(-1, 1)) == -1
    ctx.close()


def test_scheme_options_are_checked(built_lib):
    """The pitch-angle and perpendicular schemes exist only for the types that have those steps, and only
    0, 1 and 2 name a scheme."""
    ctx = capi.Context(TRAJ_PARKER, 0, 0, capi.SPX_FP64)
    assert _code(lambda: ctx.set_option(capi.SPX_OPT_PERP_METHOD, 1.0)) == capi.SPX_ERR_INVALID_ARG
    assert _code(lambda: ctx.set_option(capi.SPX_OPT_MU_METHOD, 2.0)) == capi.SPX_ERR_INVALID_ARG
    ctx.close()
    ctx = capi.Context(TRAJ_GUIDING_DIFF, 0, 25, capi.SPX_FP64)
    ctx.set_option(capi.SPX_OPT_PERP_METHOD, 2.0)
    assert _code(lambda: ctx.set_option(capi.SPX_OPT_PERP_METHOD, 3.0)) == capi.SPX_ERR_INVALID_ARG
    ctx.close()

