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
    _same_paths(gpu.records[0], ref, 1e-12)


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
    ot.assert_fp64_parity(gpu.records[0], ref, ot.run_oracle(pb, nudge_libm=1), distros=gpu.distros[0])


def test_pitch_angle_isotropisation(built_lib):
    """Pure pitch-angle scattering with D_mumu = D0 (1 - mu^2) relaxes a ring of pitch cosine mu0
    to isotropy: <mu> decays as mu0 exp(-2 D0 t) (benchmarks/benchmark_explained.txt:34-39). The
    ring sampler gives focused trajectories (p0, cos theta0, 0) (src/initial_momentum.cc:203-217)."""
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundUniform, BoundaryTimeExpire, DiffusionIsotropicConstant,
                                        DistributionTimeUniform, InitialMomentumRing, InitialSpaceFixed,
                                        InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, TRAJ_FOCUSED, Problem, distro_header
    d0 = 1.0
    t_end = 0.25
    theta0 = 0.3
    pb = Problem(traj=TRAJ_FOCUSED, time_flow=FORWARD, rk=25, seed=77, n_traj=40_000)
    pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0)).double(1.0e3))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumRing(), DC().double(1.0).double(theta0))
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
        expect = math.cos(theta0) * math.exp(-2.0 * d0 * t)
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


def test_batched_problems_match_oracle(built_lib):
    """A batch of problems with different diffusion coefficients in one launch: every problem's
    trajectories equal the oracle's for that problem (its problem id keys its random streams)."""
    pbs = []
    for k, kappa in enumerate((0.5, 1.0, 2.0)):
        pb = workloads.diffusion_uniform(n_traj=200, kappa=kappa, t_end=0.2)
        pb.problem_id = k
        pbs.append(pb)
    batch = run_problems(pbs, precision=capi.SPX_FP64, record=True)
    for k, pb in enumerate(pbs):
        ref = ot.run_oracle(pb)
        rec = batch.records[k]
        assert np.array_equal(rec["steps"], ref.traj["steps"])
        assert np.allclose(rec["pos"], ref.traj["pos"], rtol=1e-12, atol=1e-14)
        counts, _, nev = batch.distros[k][0]
        rc, _, rn = ref.distros[0]
        assert nev == rn and np.array_equal(counts, rc)


def test_cpp_application_equals_python_path(built_lib, tmp_path):
    """A reference-style C++ application on include/spx_simulation.hh gives, trajectory set for
    trajectory set, the spectrum the Python host path gives."""
    import os
    import shutil
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "gcr_modulation")
    lib_dir = os.path.dirname(built_lib)
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(root, "include"),
                    os.path.join(root, "spectrum_gb300", "examples", "gcr_modulation.cc"), "-L", lib_dir, "-lspx",
                    f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    n_e, n, years = 3, 2000, 0.2
    out = subprocess.run([exe, str(n_e), str(n), str(years), str(capi.SPX_MIXED), str(tmp_path / "x_")], check=True,
                         capture_output=True, text=True).stdout.split("\n")
    rows = [line.split() for line in out if line.strip()]
    pbs = workloads.gcr_modulation(n_traj=n, energies_mev=workloads.modulation_energies(n_e), t_max_years=years,
                                   pow_law_b=-1.0)
    res = run_problems(pbs, precision=capi.SPX_MIXED)
    for k in range(n_e):
        counts, sums, _ = res.distros[k][0]
        assert int(rows[k][2]) == int(counts.sum()), k
        assert math.isclose(float(rows[k][3]), float(sums[:, 0].sum()), rel_tol=1e-9), k


@pytest.mark.parametrize("precision", [capi.SPX_MIXED, capi.SPX_FP64])
def test_autotune_changes_speed_not_results(built_lib, precision):
    """spx_autotune picks a launch shape from timed samples; runs with it give the same
    trajectories as runs with the default shape (results do not depend on the schedule)."""
    from spectrum_gb300.simulation import open_problems
    pbs = workloads.gcr_modulation(n_traj=400, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    a = open_problems(pbs, precision=precision, record=True, deriv_mode=1)
    b = open_problems(pbs, precision=precision, record=True, deriv_mode=1)
    try:
        st_a = a.MainLoop()
        tuned = b.ctx.autotune(20000)
        # the candidate block sizes: 128, 64 and 32 threads (FP32), 128 and 64 (FP64)
        assert tuned.block_size in (32, 64, 128) and tuned.schedule in (0, 1)
        st_b = b.MainLoop()
        assert (st_b.tuning.block_size, st_b.tuning.steps_per_sync, st_b.tuning.schedule) == \
               (tuned.block_size, tuned.steps_per_sync, tuned.schedule)
        assert st_a.trajectories == st_b.trajectories and st_a.steps == st_b.steps
        for k, p in enumerate(pbs):
            ra, rb = a.ctx.records(k, p.n_traj), b.ctx.records(k, p.n_traj)
            for f in ("steps", "status", "t", "pos", "mom"):
                assert np.array_equal(ra[f], rb[f]), (k, f)
            ca, _, na = a.ctx.distribution(k, 0)
            cb, _, nb = b.ctx.distribution(k, 0)
            assert na == nb and np.array_equal(ca, cb)
    finally:
        a.close()
        b.close()


def test_pitch_angle_scattering_parallel_diffusion(built_lib):
    """Focused transport with isotropic scattering D_mumu = D0 (1 - mu^2) in a uniform field: the
    spread along the field is that of a diffusion with kappa_par = v^2 / (6 D0)
    (benchmarks/main_test_pa_scatt.cc:252; the standard (v^2/8) int (1-mu^2)^2 / D_mumu dmu),
    including the ballistic start, <z^2> = 2 kappa (t - tau (1 - exp(-t / tau))), tau = 1 / (2 D0)."""
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundUniform, BoundaryTimeExpire, DiffusionIsotropicConstant,
                                        DistributionTimeUniform, InitialMomentumShell, InitialSpaceFixed,
                                        InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, TRAJ_FOCUSED, Problem, distro_header
    d0, t_end, p0 = 1.0, 20.0, 1.0
    pb = Problem(traj=TRAJ_FOCUSED, time_flow=FORWARD, rk=25, seed=91, n_traj=20_000)
    pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0)).double(1.0e3))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumShell(), DC().double(p0))
    pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(d0))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(t_end))
    c = distro_header(DC(), (4, 0, 0), (0.0, 0, 0), (t_end * 1.01, 0, 0))
    c.double(1.0).double(0.0).int(1)
    pb.AddDistribution(DistributionTimeUniform(), c)
    pb.options[workloads.SPX_OPT_PA_SCATTERING] = 1.0
    v = units.Vel(p0)
    kappa = v * v / (6.0 * d0)
    tau = 1.0 / (2.0 * d0)
    for prec in (capi.SPX_MIXED, capi.SPX_FP64):
        rec = run_problems(pb, precision=prec, record=True).records[0]
        t = rec["t"].mean()
        z2 = (rec["pos"][:, 2] ** 2).mean()
        expect = 2.0 * kappa * (t - tau * (1.0 - math.exp(-t / tau)))
        assert abs(z2 / expect - 1.0) < 0.05, (prec, z2, expect)


def test_dipole_drift_period(built_lib):
    """10 MeV protons at L = 4 with 90 degree pitch drift westward around the dipole with the period
    3600 s * 1.05 / (E_MeV L (1 + 0.43 sin theta_eq)) of the reference's benchmark
    (benchmarks/main_test_dipole_periods.cc:129): after a quarter period the azimuth, averaged over
    gyrophases, has turned by -pi/2 to within a few percent; |p| is conserved."""
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import InitialMomentumRing, InitialSpaceFixed, InitialTimeFixed
    from spectrum_gb300.problem import Problem
    e_mev, L = 10.0, 4.0
    t_drift = 3600.0 * 1.05 / (e_mev * L * 1.43) / units.unit_time
    src = workloads.dipole_orbits(n_traj=4000, t_end=0.25 * t_drift)
    r_e = workloads.R_EARTH_CM / units.unit_length
    pb = Problem(traj=src.traj, time_flow=src.time_flow, rk=src.rk, seed=17, n_traj=4000)
    for e in src.plugins:
        if not type(e.plugin).__name__.startswith("Initial"):
            pb.plugins.append(e)
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((L * r_e, 0.0, 0.0)))
    pb.AddInitial(InitialMomentumRing(), DC().double(units.mev_to_mom(e_mev)).double(0.5 * math.pi))
    pb.options.update(src.options)
    for prec in (capi.SPX_MIXED, capi.SPX_FP64):
        rec = run_problems(pb, precision=prec, record=True).records[0]
        phi = np.arctan2(rec["pos"][:, 1], rec["pos"][:, 0])
        frac = phi.mean() / (-0.5 * math.pi * rec["t"].mean() / (0.25 * t_drift))
        assert abs(frac - 1.0) < 0.05, (prec, phi.mean(), frac)
        p = np.linalg.norm(rec["mom"], axis=1)
        assert np.max(np.abs(p / np.linalg.norm(rec["mom0"], axis=1) - 1.0)) < 1e-4


@pytest.mark.parametrize("precision", [capi.SPX_MIXED, capi.SPX_FP64])
def test_ragged_batch_with_empty_problem(built_lib, precision):
    """Problems of 0, 1 and 1,000 trajectories in one launch: the empty problem records nothing, the
    others equal their own launches (FP64: trajectory by trajectory against the oracle)."""
    pbs = []
    for k, n in enumerate((0, 1, 1000)):
        pb = workloads.diffusion_uniform(n_traj=n, t_end=0.1)
        pb.problem_id = k
        pbs.append(pb)
    res = run_problems(pbs, precision=precision, record=True)
    assert res.stats.trajectories == 1001
    assert res.stats.events == 1001  # one distribution event per trajectory (the time boundary)
    counts0, _, nev0 = res.distros[0][0]
    assert nev0 == 0 and counts0.sum() == 0 and len(res.records[0]) == 0
    for k in (1, 2):
        counts, _, nev = res.distros[k][0]
        assert nev == pbs[k].n_traj and counts.sum() == pbs[k].n_traj
        if precision == capi.SPX_FP64:
            ref = ot.run_oracle(pbs[k])
            assert np.array_equal(res.records[k]["steps"], ref.traj["steps"])
            assert np.allclose(res.records[k]["pos"], ref.traj["pos"], rtol=1e-12, atol=1e-14)


def test_run_refuses_trajectory_ids_beyond_32_bits(built_lib):
    """Trajectory ids are 32-bit Philox counter words: a run whose ids would pass 2^32 is refused
    before anything is launched, and the context stays usable."""
    from spectrum_gb300.simulation import open_problems
    pb = workloads.diffusion_uniform(n_traj=1000, t_end=0.05)
    sim = open_problems(pb, precision=capi.SPX_FP64)
    try:
        sim.ctx.set_option(capi.SPX_OPT_RUN_INDEX, 4_294_967)  # ids up to 4,294,968,000 > 2^32
        with pytest.raises(capi.SpxError) as e:
            sim.ctx.run()
        assert e.value.code == -7  # SPX_ERR_LIMIT
        sim.ctx.set_option(capi.SPX_OPT_RUN_INDEX, 4_294_966)  # the last run that fits
        st = sim.MainLoop()
        assert st.trajectories == 1000
    finally:
        sim.close()


@pytest.mark.parametrize("workload", ["modulation", "diffusion", "guiding"])
def test_specialised_kernels_equal_the_generic_one(built_lib, workload):
    """SPX_MIXED Parker contexts run on kernels compiled for their diffusion class (RigidityMagneticField-
    PowerLaw, FullConstant) and, for the modulation set-up (a time limit and two spheres), for that
    boundary layout; SPX_OPT_SPECIALIZE 2 keeps the class only, 0 forces the kernel that dispatches at run
    time. The same trajectories, bin for bin (they differ only in the dispatch the compiler removed). The guiding-
    centre kernel without the scattering and perpendicular steps agrees to FP32 rounding (same steps and outcomes)."""
    from spectrum_gb300.simulation import open_problems
    if workload == "modulation":
        pbs = workloads.gcr_modulation(n_traj=2000, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    elif workload == "guiding":  # TrajectoryGuiding proper: the kernel without scattering and perpendicular steps
        pbs = [workloads.guiding_dipole(n_traj=2000, t_end_s=5.0)]
    else:
        pbs = [workloads.diffusion_uniform(n_traj=4000, t_end=0.2)]
    out = []
    for special in (0, 1, 2):
        sim = open_problems(pbs, precision=capi.SPX_MIXED, record=True)
        sim.ctx.set_option(capi.SPX_OPT_SPECIALIZE, float(special))
        st = sim.MainLoop()
        out.append((st, [sim.ctx.records(k, p.n_traj) for k, p in enumerate(pbs)],
                    [sim.ctx.distribution(k, 0) for k in range(len(pbs))]))
        sim.close()
    sa, ra, da = out[0]
    for sb, rb, db in out[1:]:
        assert sa.steps == sb.steps
        for x, y in zip(ra, rb):
            assert np.array_equal(x["steps"], y["steps"])
            assert np.array_equal(x["status"] & STATUS_MASK, y["status"] & STATUS_MASK)
            if workload == "guiding":
                # the kernel without the other guiding types' steps contracts some multiply-adds differently:
                # the same steps and outcomes, positions equal to FP32 rounding
                scale = np.linalg.norm(x["pos"], axis=1)
                assert (np.linalg.norm(x["pos"] - y["pos"], axis=1) / scale).max() < 1e-5
            else:
                assert np.array_equal(x["pos"], y["pos"])
        for x, y in zip(da, db):
            if workload == "guiding":
                assert x[2] == y[2] and np.abs(x[0].astype(np.int64) - y[0]).sum() <= max(2, x[2] // 1000)
            else:
                assert np.array_equal(x[0], y[0])


def test_dipole_orbits_per_trajectory_errors(built_lib):
    """Full orbits in the dipole (the reference's drift-period benchmark set-up) from identical initial
    conditions, trajectory by trajectory: the FP64 kernel against the oracle at the libm level, and the
    FP32 kernel against FP64 -- relative |p| difference, azimuth (drift phase) difference and the
    difference of the energy drifts |p|/|p0| - 1, which RK4 truncation dominates in both."""
    pb = workloads.dipole_orbits(n_traj=512, t_end=1.0 / units.unit_time)
    r64 = run_problems(pb, precision=capi.SPX_FP64, record=True).records[0]
    r32 = run_problems(pb, precision=capi.SPX_MIXED, record=True).records[0]
    ot.assert_fp64_parity(r64, ot.run_oracle(pb), ot.run_oracle(pb, nudge_libm=1))
    same = (r64["status"] & STATUS_MASK) == (r32["status"] & STATUS_MASK)
    assert same.mean() >= 0.99
    p0 = np.linalg.norm(r64["mom0"], axis=1)
    p64, p32 = np.linalg.norm(r64["mom"], axis=1), np.linalg.norm(r32["mom"], axis=1)
    rel = np.abs(p32 / p64 - 1.0)[same]
    assert np.median(rel) < 1e-6 and rel.max() < 1e-4, (np.median(rel), rel.max())
    az = lambda r: np.arctan2(r["pos"][:, 1], r["pos"][:, 0])  # noqa: E731
    daz = np.abs(np.angle(np.exp(1j * (az(r32) - az(r64)))))[same]
    assert np.median(daz) < 1e-5 and np.percentile(daz, 99) < 1e-3, (np.median(daz), np.percentile(daz, 99))
    ddrift = np.abs(np.abs(p32 / p0 - 1.0) - np.abs(p64 / p0 - 1.0))[same]
    assert np.median(ddrift) < 1e-6, np.median(ddrift)
