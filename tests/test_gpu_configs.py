"""GPU checks of the other workload families: Lorentz orbits and focused transport trajectory by
trajectory against the oracle (FP64) and against the FP64 kernel (FP32), the known answers of
the reference's benchmarks (diffusive-shock index, pitch-angle isotropisation), and the batched
launch against separate launches."""
import math

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import capi, units, workloads
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu

STATUS_MASK = 0x1F0


def _dipole(n_traj, t_end_s=0.5):
    """Dipole orbits from a fixed equatorial point at L = 4, isotropic 10 MeV protons."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    pb = mg._dipole_reference_classes(n_traj)
    # keep the golden set-up's plugins but stretch the time limit
    return pb


def _same_paths(rec, ref, rtol):
    assert np.array_equal(rec["steps"], ref.traj["steps"])
    assert np.array_equal(rec["status"] & STATUS_MASK, ref.traj["status"] & STATUS_MASK)
    for f in ("pos", "mom"):
        scale = np.maximum(np.linalg.norm(ref.traj[f], axis=1), 1e-300)
        err = np.linalg.norm(rec[f] - ref.traj[f], axis=1) / scale
        assert err.max() < rtol, (f, err.max())


def test_lorentz_fp64_matches_oracle(built_lib):
    pb = _dipole(64)
    gpu = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    _same_paths(gpu.records[0], ref, 1e-9)


def test_lorentz_fp32_orbits_and_energy(built_lib):
    """FP32 RK4 with float-float accumulation: the same orbits as FP64 over a few gyroperiods and
    |p| conserved (the dipole has no electric field)."""
    pb = _dipole(256)
    r64 = run_problems(pb, precision=capi.SPX_FP64, record=True).records[0]
    r32 = run_problems(pb, precision=capi.SPX_MIXED, record=True).records[0]
    p0 = np.linalg.norm(r32["mom0"], axis=1)
    drift = np.abs(np.linalg.norm(r32["mom"], axis=1) / p0 - 1.0)
    assert drift.max() < 1e-4, drift.max()
    same = r32["steps"] == r64["steps"]
    assert same.mean() > 0.9
    err = np.linalg.norm(r32["pos"] - r64["pos"], axis=1) / np.linalg.norm(r64["pos"], axis=1)
    assert np.median(err[same]) < 1e-3, np.median(err[same])


def _focused(n_traj, scattering):
    pb = workloads.focused_transport(n_problems=1, n_traj=n_traj, t_max_hours=0.5)[0]
    pb.options[workloads.SPX_OPT_PA_SCATTERING] = 1.0 if scattering else 0.0
    return pb


@pytest.mark.parametrize("scattering", [False, True])
def test_focused_fp64_matches_oracle(built_lib, scattering):
    pb = _focused(64, scattering)
    gpu = run_problems(pb, precision=capi.SPX_FP64, record=True)
    ref = ot.run_oracle(pb)
    rec = gpu.records[0]
    agree = rec["steps"] == ref.traj["steps"]
    assert agree.mean() >= 0.9, agree.mean()
    err = np.linalg.norm(rec["pos"] - ref.traj["pos"], axis=1) / np.linalg.norm(ref.traj["pos"], axis=1)
    assert np.median(err[agree]) < 1e-9


def test_pitch_angle_isotropisation(built_lib):
    """Pure pitch-angle scattering with D_mumu = D0 (1 - mu^2) relaxes a beam to isotropy:
    <mu> decays as exp(-2 D0 t) (benchmarks/benchmark_explained.txt:34-39)."""
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundUniform, BoundaryTimeExpire, DiffusionIsotropicConstant,
                                        DistributionTimeUniform, InitialMomentumBeam, InitialSpaceFixed,
                                        InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, TRAJ_FOCUSED, Problem, distro_header
    d0 = 1.0
    t_end = 0.25
    pb = Problem(traj=TRAJ_FOCUSED, time_flow=FORWARD, rk=25, seed=77, n_traj=40_000)
    pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0)).double(1.0e3))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumBeam(), DC().double(1.0))
    pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(d0))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(t_end))
    c = distro_header(DC(), (4, 0, 0), (0.0, 0, 0), (1.0, 0, 0))
    c.double(1.0).double(0.0).int(1)
    pb.AddDistribution(DistributionTimeUniform(), c)
    pb.options[workloads.SPX_OPT_PA_SCATTERING] = 1.0
    for prec in (capi.SPX_FP64, capi.SPX_MIXED):
        rec = run_problems(pb, precision=prec, record=True).records[0]
        mu = rec["mom"][:, 1]
        t = rec["t"].mean()
        expect = math.exp(-2.0 * d0 * t)
        sigma = mu.std() / math.sqrt(len(mu))
        assert abs(mu.mean() - expect) < 4.0 * sigma + 0.01, (prec, mu.mean(), expect)
        assert np.all(np.abs(mu) <= 1.0)


def test_shock_acceleration_index(built_lib):
    """Diffusive shock acceleration at a compression-4 shock: the momenta at which particles leave
    follow dN/dln p ~ p^(3 - q), q = 3s/(s - 1) = 4 (benchmarks/main_postprocess_diff_shock_acc.cc:22-36).
    The downstream escape plane sits at x = 40 so that returns from beyond it are negligible
    (exp(-U2 L / kappa) = exp(-10))."""
    pb = workloads.shock_acceleration(n_traj=40_000, x_downstream=40.0, p_max=1.0e3)
    res = run_problems(pb, precision=capi.SPX_MIXED, record=True)
    p = res.records[0]["mom"][:, 0]
    lo, hi = 2.0, 60.0
    edges = np.exp(np.linspace(math.log(lo), math.log(hi), 9))
    h, _ = np.histogram(p, bins=edges)
    x = 0.5 * (np.log(edges[1:]) + np.log(edges[:-1]))
    ok = h > 20
    slope, _ = np.polyfit(x[ok], np.log(h[ok]), 1, w=np.sqrt(h[ok]))
    assert abs(slope - (3.0 - 4.0)) < 0.12, slope


def test_batched_problems_equal_separate_runs(built_lib):
    """A batch of problems in one launch gives each problem exactly what its own launch gives
    (trajectory ids and problem ids key the random streams)."""
    pbs = workloads.gcr_modulation(n_traj=128, energies_mev=[50.0, 500.0, 5000.0], t_max_years=0.1)
    batch = run_problems(pbs, precision=capi.SPX_FP64, record=True)
    for k, pb in enumerate(pbs):
        alone = run_problems(pb, precision=capi.SPX_FP64, record=True)
        a, b = batch.records[k], alone.records[0]
        assert np.array_equal(a["steps"], b["steps"])
        assert np.array_equal(a["pos"], b["pos"])
        ca, _, na = batch.distros[k][0]
        cb, _, nb = alone.distros[0][0]
        assert na == nb and np.array_equal(ca, cb)
