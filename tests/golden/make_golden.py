"""Generate the golden fixtures of this directory from the reference's own code.

Each fixture holds one problem spec (the exact bytes the reference harness and the oracle read),
the options the comparison needs, and the reference's output for it: per-trajectory final states
and the distributions (stored sparse). The outputs come from oracle/_ref/ref_* -- the reference's
trajectory, background, diffusion, boundary, initial and distribution sources compiled
unchanged with the Philox stand-in for GSL (oracle/Makefile, target "ref"). The reference
sources must be present to run this script; the fixtures it writes are then used everywhere,
including where the sources are not.

    python tests/golden/make_golden.py          # rewrites tests/golden/*.npz
    python tests/golden/make_golden.py NAME...  # rewrites the named fixtures only
    python tests/golden/make_golden.py --dumps  # rewrites tests/golden/*.distro<d>.out
    python tests/golden/make_golden.py --grid   # rewrites tests/golden/grid_blocks_ref.npz
    python tests/golden/make_golden.py --prints # rewrites tests/golden/distro_prints_ref.npz

The second form keeps the reference's own distribution dump files (DistributionTemplated::Dump)
of the fixtures whose distributions have at most DUMP_MAX_BINS bins: the pins of the dump format.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from spectrum_gb300 import workloads  # noqa: E402
from spectrum_gb300.workloads import SPX_OPT_MU_METHOD, SPX_OPT_PA_SCATTERING, SPX_OPT_STEPS_PER_ORBIT  # noqa: E402


def _dipole_reference_classes(n_traj: int):
    """The dipole workload's background and boundaries with initial conditions the reference
    itself provides (a fixed point at L = 4 on the equator, an isotropic 10 MeV shell)."""
    from spectrum_gb300 import units as U
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import InitialMomentumShell, InitialSpaceFixed, InitialTimeFixed
    from spectrum_gb300.problem import Problem
    src = workloads.dipole_orbits(n_traj=n_traj, t_end=0.5 / U.unit_time)
    pb = Problem(traj=src.traj, time_flow=src.time_flow, rk=src.rk, seed=src.seed, n_traj=n_traj)
    r_e = workloads.R_EARTH_CM / U.unit_length
    for e in src.plugins:
        name = type(e.plugin).__name__
        if name.startswith("Initial"):
            continue
        pb.plugins.append(e)
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0)))
    pb.AddInitial(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0)))
    return pb


def _focused_reference_classes(n_traj: int):
    """Focused transport in the Parker spiral without scattering, recorded with the reference's
    own distribution and boundary classes (time-of-exit histogram at the 1 AU absorber)."""
    from spectrum_gb300 import units as U
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundSolarWind, BoundarySphereAbsorb, BoundaryTimeExpire,
                                        DiffusionIsotropicConstant, DistributionTimeUniform, InitialMomentumShell,
                                        InitialSpaceFixed, InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, TRAJ_FOCUSED, Problem, distro_header
    au = workloads.ONE_AU
    t_max = 3600.0 / U.unit_time
    pb = Problem(traj=TRAJ_FOCUSED, time_flow=FORWARD, rk=25, seed=workloads.SEED_BASE + 5, n_traj=n_traj)
    pb.AddBackground(BackgroundSolarWind(), workloads.solarwind_params(DC()))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0.1 * au, 0, 0)))
    pb.AddInitial(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0)))
    pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(1.0e-3))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [-1]).double(t_max))
    pb.AddBoundary(BoundarySphereAbsorb(), workloads._boundary(DC(), 1, [0]).vec((0, 0, 0)).double(0.05 * au))
    pb.AddBoundary(BoundarySphereAbsorb(), workloads._boundary(DC(), 1, [0]).vec((0, 0, 0)).double(1.0 * au))
    c = distro_header(DC(), (32, 0, 0), (0.0, 0, 0), (t_max, 0, 0), bin_outside=(1, 0, 0),
                      unit_val=(U.unit_time, 1.0, 1.0))
    c.double(1.0).double(0.0).int(1)
    pb.AddDistribution(DistributionTimeUniform(), c)
    return pb


def _guiding_dipole(n_traj: int):
    """Guiding-centre orbits (TrajectoryGuiding) in the dipole: 10 MeV protons from L = 4 on the
    equator, 60 s (most of a drift period). The momentum distribution at the time boundary is
    binned in (|p|, mu) and every mirror point is an event of a time histogram (BoundaryMirror)."""
    from spectrum_gb300 import units as U
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundDipole, BoundaryMirror, BoundarySphereAbsorb, BoundaryTimeExpire,
                                        DistributionMomentumUniform, DistributionTimeUniform, InitialMomentumShell,
                                        InitialSpaceFixed, InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, TRAJ_GUIDING, Problem, distro_header
    r_e = workloads.R_EARTH_CM / U.unit_length
    b_eq = workloads.B_EARTH_G / U.unit_magnetic
    t_end = 60.0 / U.unit_time
    p0 = U.mev_to_mom(10.0)
    pb = Problem(traj=TRAJ_GUIDING, time_flow=FORWARD, rk=25, seed=workloads.SEED_BASE + 7, n_traj=n_traj)
    c = DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
    pb.AddBackground(BackgroundDipole(), c.double(r_e).double(0.1))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0)))
    pb.AddInitial(InitialMomentumShell(), DC().double(p0))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0, -1]).double(t_end))
    pb.AddBoundary(BoundarySphereAbsorb(), workloads._boundary(DC(), 1, [-1, -1]).vec((0, 0, 0)).double(r_e))
    pb.AddBoundary(BoundaryMirror(), workloads._boundary(DC(), -1, [-1, 0]))
    c = distro_header(DC(), (16, 20, 0), (0.5 * p0, -1.0, 0.0), (1.5 * p0, 1.0, 1.0))
    pb.AddDistribution(DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(1))
    c = distro_header(DC(), (60, 0, 0), (0.0, 0, 0), (t_end, 0, 0))
    pb.AddDistribution(DistributionTimeUniform(), c.double(1.0).double(0.0).int(1))
    return pb


def _slab_between_mirrors(traj: int, n_traj: int, d0: float = 0.0, keep_records: bool = False):
    """A uniform field along x between two reflecting planes at x = -1 and x = +1 (code units):
    10 MeV protons from the origin, isotropic, 5 time units (several crossings of the slab). The
    pitch-angle cosine at the time boundary is binned. With ``d0`` the pitch angle scatters with
    D_mumu = d0 (1 - mu^2) (DiffusionIsotropicConstant). With ``keep_records`` the distribution also
    keeps the value and weight of every event (DistributionTemplated::AddRecord)."""
    from spectrum_gb300 import units as U
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundUniform, BoundaryPlaneReflect, BoundaryTimeExpire,
                                        DiffusionIsotropicConstant, DistributionMomentumUniform, InitialMomentumShell,
                                        InitialSpaceFixed, InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, Problem, distro_header
    pb = Problem(traj=traj, time_flow=FORWARD, rk=25, seed=workloads.SEED_BASE + 8, n_traj=n_traj)
    pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((1.0, 0.0, 0.0)).double(0.1))
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DC().vec((0.0, 0.0, 0.0)))
    pb.AddInitial(InitialMomentumShell(), DC().double(U.mev_to_mom(10.0)))
    if d0 > 0.0:
        pb.AddDiffusion(DiffusionIsotropicConstant(), DC().double(d0))
    pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(5.0))
    pb.AddBoundary(BoundaryPlaneReflect(), workloads._boundary(DC(), -1, [-1]).vec((1.0, 0, 0)).vec((1.0, 0, 0)))
    pb.AddBoundary(BoundaryPlaneReflect(), workloads._boundary(DC(), -1, [-1]).vec((-1.0, 0, 0)).vec((-1.0, 0, 0)))
    c = distro_header(DC(), (0, 20, 0), (0.0, -1.0, 0.0), (1.0, 1.0, 1.0), keep_records=keep_records)
    pb.AddDistribution(DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(1))
    return pb


def _guiding_perp(traj: int, n_traj: int, dipole: bool):
    """Guiding centres with perpendicular diffusion (TrajectoryGuidingDiff, or GuidingDiffScatt).
    In a uniform field along x with constant D_perp = 0.05 the positions spread across the field
    (binned in y); in the dipole a rigidity and |B| power law (kappa_perp = 0.01 kappa_par ~ B)
    adds the perpendicular drift of its gradient. (With kappa ~ 1/B ~ r^3 the guiding centres would
    run away outward within seconds.)"""
    from spectrum_gb300 import units as U
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import (BackgroundDipole, BackgroundUniform, BoundarySphereAbsorb, BoundaryTimeExpire,
                                        DiffusionPerpConstant, DiffusionRigidityMagneticFieldPowerLaw,
                                        DistributionPositionUniform, InitialMomentumShell, InitialSpaceFixed,
                                        InitialTimeFixed)
    from spectrum_gb300.problem import FORWARD, Problem, distro_header
    p0 = U.mev_to_mom(10.0)
    pb = Problem(traj=traj, time_flow=FORWARD, rk=25, seed=workloads.SEED_BASE + 10, n_traj=n_traj)
    pb.AddInitial(InitialTimeFixed(), DC().double(0.0))
    pb.AddInitial(InitialMomentumShell(), DC().double(p0))
    if dipole:
        r_e = workloads.R_EARTH_CM / U.unit_length
        b_eq = workloads.B_EARTH_G / U.unit_magnetic
        c = DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
        pb.AddBackground(BackgroundDipole(), c.double(r_e).double(0.1))
        pb.AddInitial(InitialSpaceFixed(), DC().vec((4.0 * r_e, 0.0, 0.0)))
        pb.AddDiffusion(DiffusionRigidityMagneticFieldPowerLaw(),
                        DC().double(0.2).double(U.Rigidity(p0)).double(b_eq / 64.0).double(0.5).double(1.0).double(0.01))
        t_end = 30.0 / U.unit_time
        pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(t_end))
        pb.AddBoundary(BoundarySphereAbsorb(), workloads._boundary(DC(), 1, [-1]).vec((0, 0, 0)).double(r_e))
        c = distro_header(DC(), (0, 0, 20), (0, 0, -2.0 * r_e), (1, 1, 2.0 * r_e))
    else:
        pb.AddBackground(BackgroundUniform(), DC().double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((1.0, 0.0, 0.0)).double(0.1))
        pb.AddInitial(InitialSpaceFixed(), DC().vec((0.0, 0.0, 0.0)))
        pb.AddDiffusion(DiffusionPerpConstant(), DC().double(0.05))
        pb.AddBoundary(BoundaryTimeExpire(), workloads._boundary(DC(), 1, [0]).double(2.0))
        c = distro_header(DC(), (0, 20, 0), (0, -1.0, 0), (1, 1.0, 1))
    pb.AddDistribution(DistributionPositionUniform(), c.double(1.0).double(0.0).int(1).int(0))
    return pb


def cases():
    """(name, problem) pairs, each small enough for the oracle to finish in seconds."""
    out = []
    out.append(("parker_fwd_uniform", workloads.diffusion_uniform(n_traj=200)))
    dsa = workloads.shock_acceleration(n_traj=12, x_escape=-2.0, x_downstream=2.0, p_max=20.0)
    out.append(("parker_fwd_smoothshock", dsa))
    for k, pb in enumerate(workloads.gcr_modulation(n_traj=6, energies_mev=[30.0, 3000.0], t_max_years=0.05,
                                                              pow_law_b=-1.0)):
        out.append((f"parker_bwd_solarwind_{k}", pb))
    out.append(("lorentz_fwd_dipole", _dipole_reference_classes(6)))
    out.append(("focused_fwd_solarwind", _focused_reference_classes(6)))
    from spectrum_gb300.problem import TRAJ_FOCUSED, TRAJ_GUIDING_SCATT
    out.append(("focused_fwd_slab_reflect", _slab_between_mirrors(TRAJ_FOCUSED, 8)))
    out.append(("focused_fwd_slab_records", _slab_between_mirrors(TRAJ_FOCUSED, 12, keep_records=True)))
    out.append(("guiding_fwd_dipole", _guiding_dipole(6)))
    out.append(("guidingscatt_fwd_slab_reflect", _slab_between_mirrors(TRAJ_GUIDING_SCATT, 8, d0=0.5)))
    for mu in (1, 2):  # the Milstein and RK2 pitch-angle schemes (STOCHASTIC_METHOD_MU)
        pb = _slab_between_mirrors(TRAJ_GUIDING_SCATT, 8, d0=0.5)
        pb.options[SPX_OPT_MU_METHOD] = mu
        out.append((f"guidingscatt_mu{mu}_fwd_slab_reflect", pb))
    from spectrum_gb300.problem import TRAJ_GUIDING_DIFF, TRAJ_GUIDING_DIFF_SCATT
    out.append(("guidingdiff_fwd_uniform", _guiding_perp(TRAJ_GUIDING_DIFF, 8, dipole=False)))
    out.append(("guidingdiff_fwd_dipole", _guiding_perp(TRAJ_GUIDING_DIFF, 6, dipole=True)))
    out.append(("guidingdiffscatt_fwd_uniform", _guiding_perp(TRAJ_GUIDING_DIFF_SCATT, 8, dipole=False)))
    return out


def sparse(distros):
    out = {}
    for d, (counts, sums, nev) in enumerate(distros):
        nz = np.nonzero(counts)[0]
        out[f"d{d}_n_bins"] = np.int64(len(counts))
        out[f"d{d}_width"] = np.int64(sums.shape[1])
        out[f"d{d}_idx"] = nz.astype(np.int64)
        out[f"d{d}_counts"] = counts[nz].astype(np.int32)
        out[f"d{d}_sums"] = sums[nz].astype(np.float64)
        out[f"d{d}_n_events"] = np.int64(nev)
    out["n_distros"] = np.int64(len(distros))
    return out


DUMP_MAX_BINS = 4096


def write_dumps():
    import tempfile

    import oracle_tools as ot
    for name, pb in cases():
        with tempfile.TemporaryDirectory() as td:
            ref = ot.run_reference(pb, dump_prefix=os.path.join(td, "distro"))
            for d, (counts, _, _) in enumerate(ref.distros):
                if len(counts) > DUMP_MAX_BINS:
                    continue
                with open(os.path.join(td, f"distro{d}.out"), "rb") as f:
                    data = f.read()
                path = os.path.join(HERE, f"{name}.distro{d}.out")
                with open(path, "wb") as f:
                    f.write(data)
                print(f"{name}.distro{d}.out: {len(data)} bytes")


PRINT_KINDS = [f"p1d{k}{u}" for u in ("", "u") for k in range(3)] + \
    [f"p2d{a}{b}{u}" for u in ("", "u") for a, b in ((0, 1), (0, 2), (1, 2))] + ["prec", "precu"]


def write_prints():
    """The reference's text output of the same distributions (Print1D of every axis, Print2D of every
    pair, PrintRecords; code and physical units), as oracle/_ref's harness writes it beside the dumps,
    into one compressed archive: distro_prints_ref.npz, key <case>.distro<d>.<kind>."""
    import tempfile

    import oracle_tools as ot
    out = {}
    for name, pb in cases():
        with tempfile.TemporaryDirectory() as td:
            pre = os.path.join(td, "distro")
            ref = ot.run_reference(pb, dump_prefix=pre)
            for d, (counts, _, _) in enumerate(ref.distros):
                if len(counts) > DUMP_MAX_BINS:
                    continue
                for kind in PRINT_KINDS:
                    with open(f"{pre}{d}.{kind}", "rb") as f:
                        out[f"{name}.distro{d}.{kind}"] = np.frombuffer(f.read(), dtype=np.uint8)
    path = os.path.join(HERE, "distro_prints_ref.npz")
    np.savez_compressed(path, **out)
    print(f"distro_prints_ref: {len(out)} files, {os.path.getsize(path)} bytes")


def write_grid():
    """Fields and gradients of the reference's Cartesian data server (oracle/_ref/ref_grid0) at the
    probe points of tests/test_oracle_grid_blocks.py, with the grid they were computed on."""
    import pathlib
    import tempfile

    import test_oracle_grid_blocks as tg
    g = tg.synthetic_grid()
    pts = tg.probe_points(g)
    dmax0 = 0.05 * tg.AU / tg.L
    with tempfile.TemporaryDirectory() as td:
        rows = tg.run_harness(0, g, pts, dmax0, pathlib.Path(td))
    fields = np.array([[float(x) for x in r[1:]] for r in rows])
    path = os.path.join(HERE, "grid_blocks_ref.npz")
    np.savez_compressed(path, n_blocks=np.array(g.n_blocks), domain_min=np.array(g.domain_min),
                        domain_max=np.array(g.domain_max), values=g.values, points=pts, fields=fields,
                        status=np.array([int(r[0]) for r in rows]), dmax0=np.float64(dmax0))
    print(f"grid_blocks_ref: {len(pts)} points, {os.path.getsize(path)} bytes")


def main():
    args = sys.argv[1:]
    if "--dumps" in args:
        write_dumps()
        return
    if "--grid" in args:
        write_grid()
        return
    if "--prints" in args:
        write_prints()
        return
    import oracle_tools as ot
    for name, pb in cases():
        if args and name not in args:
            continue
        ref = ot.run_reference(pb)
        fx = {"spec": np.frombuffer(pb.to_spec(), dtype=np.uint8), "traj": ref.traj,
              "traj_kind": np.int64(pb.traj), "time_flow": np.int64(pb.time_flow), "rk": np.int64(pb.rk),
              "steps_per_orbit": np.float64(pb.options.get(SPX_OPT_STEPS_PER_ORBIT, 100.0)),
              "pa_scattering": np.int64(pb.options.get(SPX_OPT_PA_SCATTERING, 0)),
              "mu_method": np.int64(pb.options.get(SPX_OPT_MU_METHOD, 0)),
              "n_traj": np.int64(pb.n_traj)}
        fx.update(sparse(ref.distros))
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fx)
        print(f"{name}: {len(ref.traj)} trajectories, {int(ref.traj['steps'].sum())} steps, "
              f"{os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
