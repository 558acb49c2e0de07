"""Butcher tables beyond Euler and RK4 on the device: the FP64 kernels of any table against the
oracle, trajectory by trajectory, on the problems tests/test_oracle_rk.py pins bit for bit to the
reference compiled with each table (adaptive tables with rejected steps included). The device
follows deviation D6 (after a rejected step, the fields of the restored point), so the oracle runs
without the reference's quirk here."""
import pytest

import oracle_tools as ot
import test_oracle_rk as cases
from spectrum_gb300 import capi, workloads
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(cases.RK_CASES))
def test_table_on_device(built_lib, name):
    pb = cases.RK_CASES[name]()
    res = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    ot.assert_fp64_parity(res.records[0], ref, ot.run_oracle(pb, nudge_libm=1), distros=res.distros[0])
    assert res.stats.given_up == 0


@pytest.mark.parametrize("rk,precision", [(29, capi.SPX_MIXED), (16, capi.SPX_MIXED), (30, capi.SPX_FP64),
                                          (33, capi.SPX_FP64), (-1, capi.SPX_FP64)])
def test_unsupported_tables_are_refused(built_lib, rk, precision):
    """The general tables run in FP64 only; table 30 does not compile in the reference; others do not exist."""
    pb = workloads.diffusion_uniform(n_traj=4, t_end=0.01)
    with pytest.raises(capi.SpxError) as e:
        capi.Context(pb.traj, pb.time_flow, rk, precision)
    assert e.value.code == -1  # SPX_ERR_INVALID_ARG


def test_fixed_and_general_kernels_agree_on_rk4(built_lib):
    """Parker with the classic RK4 table runs on the general-table kernels; the same table on a Lorentz
    problem runs on the unrolled kernel. Each matches the oracle with that table."""
    import make_golden
    pb = make_golden._dipole_reference_classes(6)  # Lorentz, table 25: the unrolled kernel
    res = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ot.assert_fp64_parity(res.records[0], ot.run_oracle(pb), ot.run_oracle(pb, nudge_libm=1))
    pk = cases._with_rk(cases.cases._combo("parker_dipole"), 25)  # Parker, table 25: the general kernel
    res = run_problems(pk, precision=capi.SPX_FP64, record=True)
    ot.assert_fp64_parity(res.records[0], ot.run_oracle(pk), ot.run_oracle(pk, nudge_libm=1), distros=res.distros[0])
