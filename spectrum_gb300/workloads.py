"""The five benchmark workloads, set up the way a reference user would set them up.

Each builder fills a ``Problem`` with ``Add*(Prototype(), DataContainer)`` calls in the order and
with the parameter layout of the reference's own mains (benchmarks/main_test_full_diff.cc:37-244,
runs/gcr_modulation_example.cc:76-332, benchmarks/main_test_dipole_periods.cc:42-72). Inputs are
synthetic; seeds are fixed (``0x5eed0000 + workload number``; problem p of a batch uses
problem id p).

  1  pure spatial diffusion        Parker fwd, uniform B, kappa = 1, t = 1, 3-D position histogram
  2  diffusive shock acceleration  Parker fwd, smooth planar shock s = 4, log-p histogram
  3  dipole Lorentz orbits         Lorentz RK4, dipole, log-uniform E, L in [2,6], pitch band
  4  GCR modulation                Parker bwd, Parker spiral, 32 energies, LIS-weighted spectrum
  5  focused transport             Focused RK4 + pitch-angle scattering, 64 problems, (t, mu)

Sizes default to the full workload; every builder takes ``n_traj`` (per problem) so tests can
shrink them.
"""
from __future__ import annotations

import math

from . import units as U
from .datacontainer import DataContainer
from .plugins import (BackgroundDipole, BackgroundSmoothShock, BackgroundSolarWind, BackgroundUniform,
                      BoundaryMirror, BoundaryMomentumInject, BoundaryPlaneAbsorb, BoundarySphereAbsorb, BoundarySpherePass,
                      BoundaryTimeExpire, DiffusionFullConstant, DiffusionIsotropicConstant,
                      DiffusionRigidityMagneticFieldPowerLaw, DistributionMomentumUniform,
                      DistributionPositionUniform, DistributionSpectrumKineticEnergyPowerLaw,
                      DistributionTimeMu, DistributionTimeUniform, InitialMomentumLogEnergyPitchBand,
                      InitialMomentumShell, InitialSpaceEquatorialBand, InitialSpaceFixed, InitialTimeFixed)
from .problem import BACKWARD, FORWARD, TRAJ_FOCUSED, TRAJ_GUIDING, TRAJ_LORENTZ, TRAJ_PARKER, Problem, distro_header

ONE_AU = U.ASTRONOMICAL_UNIT / U.unit_length
SEED_BASE = 0x5EED0000


def _boundary(c: DataContainer, max_crossings: int, actions) -> DataContainer:
    """BoundaryBase header: int max_crossings, std::vector<int> actions (src/boundary_base.cc:138-141)."""
    return c.int(max_crossings).ints(actions)


# ------------------------------------------------------------------------------------------------
# 1. pure spatial diffusion
# ------------------------------------------------------------------------------------------------
def diffusion_uniform(n_traj: int = 100_000, kappa: float = 1.0, t_end: float = 1.0, dt: float = 1.0e-3,
                      n_bins: int = 100, half_width: float = 6.0) -> Problem:
    """Parker forward, uniform B along z, U = 0, constant isotropic kappa.

    dt is not an input of the reference: it is min(dt_physical, dt_adaptive) with the diffusive
    bound 0.5 * dmax^2 / max(kappa) (src/trajectory_parker.cc:212-221). dmax0 is therefore chosen
    as sqrt(2 * kappa * dt) so that the step is ``dt``.
    """
    pb = Problem(traj=TRAJ_PARKER, time_flow=FORWARD, rk=0, seed=SEED_BASE + 1, n_traj=n_traj)
    dmax0 = math.sqrt(2.0 * kappa * dt)
    c = DataContainer()
    c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, 1.0)).double(dmax0)
    pb.AddBackground(BackgroundUniform(), c)
    pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DataContainer().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumShell(), DataContainer().double(1.0))
    pb.AddDiffusion(DiffusionFullConstant(), DataContainer().double(kappa).double(kappa))
    pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [0]).double(t_end))
    c = distro_header(DataContainer(), (n_bins,) * 3, (-half_width,) * 3, (half_width,) * 3)
    c.double(1.0).double(0.0).int(1).int(0)        # val_hot, val_cold, val_time, val_coord
    pb.AddDistribution(DistributionPositionUniform(), c)
    return pb


# ------------------------------------------------------------------------------------------------
# 2. diffusive shock acceleration
# ------------------------------------------------------------------------------------------------
def shock_acceleration(n_traj: int = 10_000_000, s: float = 4.0, u1: float = 1.0, kappa: float = 1.0,
                       width_frac: float = 1.0e-3, p_max: float = 1.0e3, x_escape: float = -10.0,
                       x_downstream: float = 10.0, n_bins: int = 200, dmax_fraction: float = 0.1) -> Problem:
    """Parker forward in a smooth planar shock; injection at the shock with p0 = 1.

    The shock normal points upstream (-x): the flow u0 = (U1, 0, 0) enters from x < 0 and is
    compressed by ``s`` behind the shock at x = 0 (src/background_shock.cc:58-80). The width is
    ``width_frac`` of the diffusion length kappa/U1. Trajectories end at the momentum boundary
    p_max (recorded), at the free-escape plane x = x_escape upstream, or at the downstream
    escape plane x = x_downstream (both recorded with their own action so the spectrum can be
    formed from the momentum reached). The recorded value is p at termination.
    """
    pb = Problem(traj=TRAJ_PARKER, time_flow=FORWARD, rk=0, seed=SEED_BASE + 2, n_traj=n_traj)
    width = width_frac * kappa / u1
    dmax0 = 0.05 * kappa / u1
    c = DataContainer()
    c.double(0.0).vec((0, 0, 0)).vec((u1, 0, 0)).vec((1.0, 0.0, 0.0)).double(dmax0)
    c.vec((-1.0, 0.0, 0.0)).double(0.0).double(s)          # n_shock, v_shock, compression
    c.double(width).double(dmax_fraction)                  # width_shock, dmax_fraction
    pb.AddBackground(BackgroundSmoothShock(), c)
    pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
    pb.AddInitial(InitialSpaceFixed(), DataContainer().vec((0, 0, 0)))
    pb.AddInitial(InitialMomentumShell(), DataContainer().double(1.0))
    pb.AddDiffusion(DiffusionFullConstant(), DataContainer().double(kappa).double(kappa))
    pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [-1]).double(1.0e6 * kappa / u1 ** 2))
    pb.AddBoundary(BoundaryPlaneAbsorb(), _boundary(DataContainer(), 1, [0]).vec((x_escape, 0, 0)).vec((-1, 0, 0)))
    pb.AddBoundary(BoundaryPlaneAbsorb(), _boundary(DataContainer(), 1, [0]).vec((x_downstream, 0, 0)).vec((1, 0, 0)))
    pb.AddBoundary(BoundaryMomentumInject(), _boundary(DataContainer(), 1, [0]).double(p_max))
    c = distro_header(DataContainer(), (n_bins, 0, 0), (1.0, 0, 0), (p_max * 1.0000001, 0, 0), log_bins=(1, 0, 0),
                      bin_outside=(1, 0, 0))
    c.double(1.0).double(0.0).int(1).int(0)                # val_hot, val_cold, val_time, val_coord
    pb.AddDistribution(DistributionMomentumUniform(), c)
    return pb


# ------------------------------------------------------------------------------------------------
# 3. Lorentz orbits in a dipole
# ------------------------------------------------------------------------------------------------
R_EARTH_CM = 6.37e8
B_EARTH_G = 0.311


def dipole_orbits(n_traj: int = 1_000_000, e1_mev: float = 1.0, e2_mev: float = 100.0, l1: float = 2.0,
                  l2: float = 6.0, pitch_deg=(10.0, 170.0), steps_per_orbit: int = 32,
                  n_drift_periods: float = 100.0, t_end: float | None = None) -> Problem:
    """Full orbits in an Earth-like dipole (benchmarks/main_test_dipole_periods.cc:42-72).

    The drift-period scale of the slowest particle (1 MeV at L = 2) sets the default time limit
    of ``n_drift_periods`` periods; ``t_end`` overrides it (tests use a few gyroperiods).
    """
    pb = Problem(traj=TRAJ_LORENTZ, time_flow=FORWARD, rk=25, seed=SEED_BASE + 3, n_traj=n_traj)
    r_e = R_EARTH_CM / U.unit_length
    b_eq = B_EARTH_G / U.unit_magnetic
    c = DataContainer()
    c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
    c.double(r_e).double(0.1)                              # r_ref, dmax_fraction
    pb.AddBackground(BackgroundDipole(), c)
    pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
    pb.AddInitial(InitialSpaceEquatorialBand(), DataContainer().vec((0, 0, 0)).double(r_e).double(l1).double(l2))
    mu_lo = math.cos(math.radians(pitch_deg[1]))
    mu_hi = math.cos(math.radians(pitch_deg[0]))
    pb.AddInitial(InitialMomentumLogEnergyPitchBand(),
                  DataContainer().double(e1_mev * U.MEV / U.unit_energy).double(e2_mev * U.MEV / U.unit_energy)
                  .double(mu_lo).double(mu_hi))
    if t_end is None:
        # drift period (s) ~ 3600*1.05/(E_MeV * L * (1+0.43)) for equatorial pitch
        # (benchmarks/main_test_dipole_periods.cc:129-130)
        t_drift = 3600.0 * 1.05 / (e1_mev * l1 * 1.43) / U.unit_time
        t_end = n_drift_periods * t_drift
    pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [0]).double(t_end))
    pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [1]).vec((0, 0, 0)).double(r_e))
    c = distro_header(DataContainer(), (64, 32, 0), (e1_mev * U.MEV / U.unit_energy * 0.5, -1.0, 0.0),
                      (e2_mev * U.MEV / U.unit_energy * 2.0, 1.0, 1.0), log_bins=(1, 0, 0), bin_outside=(1, 1, 0))
    c.double(1.0).double(0.0).int(1).int(1)
    pb.AddDistribution(DistributionMomentumUniform(), c)
    pb.options[SPX_OPT_STEPS_PER_ORBIT] = float(steps_per_orbit)
    return pb


def guiding_dipole(n_traj: int = 1_000_000, e1_mev: float = 1.0, e2_mev: float = 100.0, l1: float = 2.0,
                   l2: float = 6.0, pitch_deg=(10.0, 170.0), t_end_s: float = 60.0) -> Problem:
    """Trapped protons as guiding centres (TrajectoryGuiding) in the Earth-like dipole of
    ``dipole_orbits``: the same energies, L shells and pitch angles, followed for ``t_end_s``
    seconds of bounce and drift motion. The (|p|, mu) distribution at the time boundary is binned,
    and every mirror point (BoundaryMirror) is an event of a time histogram."""
    pb = Problem(traj=TRAJ_GUIDING, time_flow=FORWARD, rk=25, seed=SEED_BASE + 9, n_traj=n_traj)
    r_e = R_EARTH_CM / U.unit_length
    b_eq = B_EARTH_G / U.unit_magnetic
    t_end = t_end_s / U.unit_time
    c = DataContainer()
    c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0.0, 0.0, -b_eq)).double(0.1 * r_e)
    c.double(r_e).double(0.1)
    pb.AddBackground(BackgroundDipole(), c)
    pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
    pb.AddInitial(InitialSpaceEquatorialBand(), DataContainer().vec((0, 0, 0)).double(r_e).double(l1).double(l2))
    mu_lo = math.cos(math.radians(pitch_deg[1]))
    mu_hi = math.cos(math.radians(pitch_deg[0]))
    e1, e2 = e1_mev * U.MEV / U.unit_energy, e2_mev * U.MEV / U.unit_energy
    pb.AddInitial(InitialMomentumLogEnergyPitchBand(), DataContainer().double(e1).double(e2).double(mu_lo).double(mu_hi))
    pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [0, -1]).double(t_end))
    pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [-1, -1]).vec((0, 0, 0)).double(r_e))
    pb.AddBoundary(BoundaryMirror(), _boundary(DataContainer(), -1, [-1, 0]))
    c = distro_header(DataContainer(), (64, 32, 0), (0.5 * e1, -1.0, 0.0), (2.0 * e2, 1.0, 1.0), log_bins=(1, 0, 0),
                      bin_outside=(1, 1, 0))
    pb.AddDistribution(DistributionMomentumUniform(), c.double(1.0).double(0.0).int(1).int(1))
    c = distro_header(DataContainer(), (60, 0, 0), (0.0, 0, 0), (t_end, 0, 0))
    pb.AddDistribution(DistributionTimeUniform(), c.double(1.0).double(0.0).int(1))
    return pb


# ------------------------------------------------------------------------------------------------
# 4. GCR modulation in the Parker spiral (backward in time)
# ------------------------------------------------------------------------------------------------
def solarwind_params(c: DataContainer, dmax0: float = ONE_AU) -> DataContainer:
    """BackgroundSolarWind container of runs/gcr_modulation_example.cc:40-78: 400 km/s radial wind,
    |B| = 5 nT at 1 AU scaled from r_ref = 3 solar radii, 25-day rotation about +z."""
    umag = 4.0e7 / U.unit_velocity
    rs = 6.957e10 / U.unit_length
    r_ref = 3.0 * rs
    bmag_e = 5.0e-5 / U.unit_magnetic
    bmag_ref = bmag_e * (ONE_AU / r_ref) ** 2
    w0 = 2.0 * math.pi / (25.0 * 24.0 * 3600.0) * U.unit_time
    c.double(0.0).vec((0, 0, 0)).vec((umag, 0, 0)).vec((bmag_ref, 0, 0)).double(dmax0)
    c.vec((0.0, 0.0, w0)).double(r_ref).double(0.1)
    return c


BMAG_1AU = 5.0e-5 / U.unit_magnetic


def modulation_energies(n: int = 32, e1_mev: float = 10.0, e2_mev: float = 1.0e4) -> list[float]:
    return [e1_mev * (e2_mev / e1_mev) ** (i / (n - 1)) for i in range(n)] if n > 1 else [e1_mev]


#: span of the modulation runs' exit-time histogram (32 bins from 0 back to this many years)
T_HIST_YEARS = 10.0


def gcr_modulation(n_traj: int = 1_000_000, energies_mev=None, lam0_au: float = 0.1, pow_law_r: float = 0.5,
                   pow_law_b: float = 0.0, kap_rat: float = 0.02, r_inner_au: float = 0.05,
                   r_outer_au: float = 100.0, t_max_years: float = 100.0, lis_gamma: float = -1.8,
                   t_hist_years: float = T_HIST_YEARS) -> list[Problem]:
    """One problem per energy: start at 1 AU, trace backward until the 100 AU outer boundary
    (hot: weighted by the LIS J0 (T/T0)^gamma / p^2 * v, src/distribution_other.cc:553-602) or the
    0.05 AU inner boundary (cold).

    kappa_par = (lam0 v / 3)(R/R0)^0.5 (B/B0)^pow_law_b, kappa_perp = kap_rat kappa_par
    (src/diffusion_other.cc:804-809). The defaults are the modulation configuration of 32 energies
    x 1e6 trajectories: lambda grows as P^0.5 with no field dependence (pow_law_b = 0). Every
    trajectory ends at one of the two spheres within about four years and 1e6 steps; the reference
    requires one time boundary (src/trajectory_base.cc:626-627), so a BoundaryTimeExpire sits
    ``t_max_years`` = 100 years back, which no trajectory reaches (its crossings are neither hot nor
    cold). The reference's run example (runs/gcr_modulation_example.cc:177-220) instead uses
    pow_law_b = -1, kap_rat = 0.05 and a limit one year back. The exit-time histogram spans the
    shorter of ``t_hist_years`` and the limit, outliers in its end bins.
    """
    if energies_mev is None:
        energies_mev = modulation_energies()
    out = []
    # (years * 365 * 24 * 3600) / unit_time, in this order: the blobs must round as the reference's mains do
    t_max = t_max_years * 365.0 * 24.0 * 3600.0 / U.unit_time
    t_hist = t_max if t_max_years <= t_hist_years else t_hist_years * 365.0 * 24.0 * 3600.0 / U.unit_time
    r0_rig = 3.33e6 / (U.unit_energy / U.unit_charge)
    unit_distro = 1.0 / (U.unit_length ** 2 * U.unit_time * 4.0 * math.pi * U.unit_energy)
    for p_idx, e in enumerate(energies_mev):
        pb = Problem(traj=TRAJ_PARKER, time_flow=BACKWARD, rk=0, seed=SEED_BASE + 4, n_traj=n_traj, problem_id=p_idx)
        pb.AddBackground(BackgroundSolarWind(), solarwind_params(DataContainer()))
        pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
        pb.AddInitial(InitialSpaceFixed(), DataContainer().vec((ONE_AU, 0, 0)))
        p0 = U.mev_to_mom(e)
        pb.AddInitial(InitialMomentumShell(), DataContainer().double(p0))
        # actions per distribution: (spectrum, exit time); the inner boundary is "cold" for the spectrum
        pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [1, -1]).vec((0, 0, 0)).double(r_inner_au * ONE_AU))
        pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [0, 0]).vec((0, 0, 0)).double(r_outer_au * ONE_AU))
        pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [-1, -1]).double(-t_max))
        pb.AddDiffusion(DiffusionRigidityMagneticFieldPowerLaw(),
                        DataContainer().double(lam0_au * ONE_AU).double(r0_rig).double(BMAG_1AU)
                        .double(pow_law_r).double(pow_law_b).double(kap_rat))
        t1 = U.EnrKin(U.mev_to_mom(energies_mev[0])) * 0.5
        t2 = U.EnrKin(U.mev_to_mom(energies_mev[-1])) * 2.0
        c = distro_header(DataContainer(), (len(energies_mev) * 4, 0, 0), (t1, 0, 0), (t2, 0, 0), log_bins=(1, 0, 0),
                          unit_distro=unit_distro, unit_val=(U.unit_energy, 1.0, 1.0))
        c.double(1.0 / unit_distro).double(1.0 * U.GEV / U.unit_energy).double(lis_gamma).double(0.0)
        pb.AddDistribution(DistributionSpectrumKineticEnergyPowerLaw(), c)
        # exit-time histogram of the run example (runs/gcr_modulation_example.cc:280-330): bins from 0
        # to the (negative) end of the histogram span, outliers into the end bins
        c = distro_header(DataContainer(), (32, 0, 0), (0.0, 0, 0), (-t_hist, 0, 0), bin_outside=(1, 0, 0),
                          unit_val=(U.unit_time, 1.0, 1.0))
        c.double(1.0).double(0.0).int(1)
        pb.AddDistribution(DistributionTimeUniform(), c)
        out.append(pb)
    return out


def lis_weights(p, lis_gamma: float = -1.8):
    """The spectrum's event weight for exit momenta ``p`` (numpy array, code units): the LIS
    J0 v (T/T0)^gamma / p^2 of DistributionSpectrumKineticEnergyPowerLaw
    (src/distribution_other.cc:567-591) with J0 = 1 / unit_distro and T0 = 1 GeV, as gcr_modulation
    sets them. Used to form per-trajectory weights from final records (Monte Carlo errors)."""
    import numpy as np
    p = np.asarray(p, dtype=np.float64)
    unit_distro = 1.0 / (U.unit_length ** 2 * U.unit_time * 4.0 * math.pi * U.unit_energy)
    mc2 = U.mass * U.c_code * U.c_code
    etot = np.sqrt(p * p + (U.mass * U.c_code) ** 2) * U.c_code
    ke = etot - mc2
    v = p * U.c_code * U.c_code / etot
    t0 = 1.0 * U.GEV / U.unit_energy
    return (1.0 / unit_distro) * v * np.power(ke / t0, lis_gamma) / (p * p)


# ------------------------------------------------------------------------------------------------
# 4b. the same modulation on a gridded background
# ------------------------------------------------------------------------------------------------
def parker_spiral_fields(x, y, z, dmax0: float = ONE_AU):
    """U and B of the Parker spiral of solarwind_params at points (x, y, z) (numpy arrays): the
    closed form U = ur r/|r|, B = A r/|r|^3 + k (|r| - r_ref)/|r|^3 (r x z), A = Br0 r_ref^2, k = A w0 / ur
    (the field of src/background_solarwind.cc:111-249 in the global frame)."""
    import numpy as np
    umag = 4.0e7 / U.unit_velocity
    rs = 6.957e10 / U.unit_length
    r_ref = 3.0 * rs
    bmag_ref = (5.0e-5 / U.unit_magnetic) * (ONE_AU / r_ref) ** 2
    w0 = 2.0 * math.pi / (25.0 * 24.0 * 3600.0) * U.unit_time
    a = bmag_ref * r_ref * r_ref
    k = a * w0 / umag
    r = np.sqrt(x * x + y * y + z * z)
    pos = np.stack([x, y, z], axis=-1)
    w = np.stack([y, -x, np.zeros_like(x)], axis=-1)  # r x z
    u = (umag / r)[..., None] * pos
    f = (r - r_ref) / r ** 3
    b = (a / r ** 3)[..., None] * pos + (k * f)[..., None] * w
    return u, b


def gcr_modulation_grid(n_traj: int = 100_000, n_nodes: int = 256, half_width_au: float = 6.0,
                        energies_mev=None, r_inner_au: float = 0.3, r_outer_au: float = 5.0,
                        t_max_years: float = 0.2, **kw) -> list[Problem]:
    """The modulation problems with the Parker spiral sampled on a uniform n^3 grid over
    [-half_width, half_width]^3 AU (BackgroundServerCartesian, first-order interpolation). An even
    node count keeps the nodes off the origin. Boundaries shrink to fit the block: outer sphere
    r_outer_au (hot), inner sphere r_inner_au (cold, a few zones from the origin)."""
    from .plugins import BackgroundServerCartesian
    from .problem import Grid
    if energies_mev is None:
        energies_mev = modulation_energies(8, 30.0, 3.0e3)
    h = half_width_au * ONE_AU
    zone = 2.0 * h / (n_nodes - 1)
    grid = Grid.sample((n_nodes,) * 3, (-h,) * 3, (zone,) * 3, parker_spiral_fields)
    pbs = gcr_modulation(n_traj=n_traj, energies_mev=energies_mev, r_inner_au=r_inner_au, r_outer_au=r_outer_au,
                         t_max_years=t_max_years, **kw)
    for pb in pbs:
        c = DataContainer()
        c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 0)).double(ONE_AU)
        pb.plugins[0] = type(pb.plugins[0])(BackgroundServerCartesian(), c.data(), c.size())
        pb.grid = grid
    return pbs


def server_unit_ratios() -> tuple:
    """The reference data server's unit conversion (spx_grid_units): Fluid/Particle ratios of
    length, velocity and magnetic field, and Fluid::c_code (common/physics.hh:18-55,
    common/specie.hh:25-64)."""
    au, c, m_p, e = 1.495978707e+13, 2.99792458e+10, 1.67262192596e-24, 4.8032044e-10
    p_vel, p_len = 0.1 * c, 1.0e10
    p_mag = (m_p * p_vel) / (e * (p_len / p_vel))
    return au / p_len, 1.0e7 / p_vel, (1.0e7 * math.sqrt(m_p * 1.0)) / p_mag, c / 1.0e7


def gcr_modulation_blocks(n_traj: int = 100_000, n_blocks: int = 16, half_width_au: float = 6.0,
                          ghost_cells: int = 0, energies_mev=None, r_inner_au: float = 0.3,
                          r_outer_au: float = 5.0, t_max_years: float = 0.2, **kw) -> list[Problem]:
    """The modulation problems with the Parker spiral held as the reference's Cartesian data server
    holds a data file: n_blocks^3 blocks of 4^3 zones over [-half_width, half_width]^3 au, the
    spiral sampled at the zone centres in fluid units (BlockGrid). Boundaries as gcr_modulation_grid."""
    from .plugins import BackgroundServerCartesian
    from .problem import BlockGrid
    if energies_mev is None:
        energies_mev = modulation_energies(8, 30.0, 3.0e3)
    len_r, vel_r, mag_r, _ = server_unit_ratios()

    def fluid_fields(x, y, z):
        u, b = parker_spiral_fields(x * len_r, y * len_r, z * len_r)
        return u / vel_r, b / mag_r

    h = half_width_au
    grid = BlockGrid.sample((n_blocks,) * 3, (-h,) * 3, (h,) * 3, fluid_fields, ghost_cells)
    pbs = gcr_modulation(n_traj=n_traj, energies_mev=energies_mev, r_inner_au=r_inner_au, r_outer_au=r_outer_au,
                         t_max_years=t_max_years, **kw)
    for pb in pbs:
        c = DataContainer()
        c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 0)).double(ONE_AU)
        pb.plugins[0] = type(pb.plugins[0])(BackgroundServerCartesian(), c.data(), c.size())
        pb.grid = grid
    return pbs


# ------------------------------------------------------------------------------------------------
# 5. focused transport with pitch-angle scattering
# ------------------------------------------------------------------------------------------------
def focused_transport(n_problems: int = 64, n_min: int = 1000, n_max: int = 1_000_000, lam_au=(0.01, 1.0),
                      e_mev=(1.0, 100.0), t_max_hours: float = 48.0, n_t: int = 256, n_mu: int = 32,
                      n_traj: int | None = None, seed_offset: int = 5) -> list[Problem]:
    """64 problems in the Parker spiral: impulsive injection at 0.1 AU, isotropic, mono-energetic
    per problem (log-uniform draw in [1, 100] MeV), mean free path log-uniform in [0.01, 1] AU,
    trajectory count log-uniform in [1e3, 1e6]; an observer sphere at 1 AU records (t, mu) of
    every crossing (256 x 32 bins). Pitch-angle scattering uses D_mumu = D0 (1 - mu^2)
    (src/diffusion_other.cc:64-79) with D0 = v / (2 lambda): then kappa_par =
    (v^2/8) int (1-mu^2)^2 / D_mumu dmu = v^2 / (6 D0), so the parallel mean free path
    3 kappa_par / v equals lambda.
    The parameters of problem p come from a fixed-seed generator so the batch is reproducible.
    """
    import random
    rnd = random.Random(SEED_BASE + seed_offset)
    out = []
    t_max = t_max_hours * 3600.0 / U.unit_time
    for p_idx in range(n_problems):
        count = int(round(math.exp(rnd.uniform(math.log(n_min), math.log(n_max)))))
        lam = math.exp(rnd.uniform(math.log(lam_au[0]), math.log(lam_au[1]))) * ONE_AU
        e = math.exp(rnd.uniform(math.log(e_mev[0]), math.log(e_mev[1])))
        p0 = U.mev_to_mom(e)
        v = U.Vel(p0)
        d0 = v / (2.0 * lam)
        pb = Problem(traj=TRAJ_FOCUSED, time_flow=FORWARD, rk=25, seed=SEED_BASE + seed_offset,
                     n_traj=n_traj if n_traj is not None else count, problem_id=p_idx)
        pb.AddBackground(BackgroundSolarWind(), solarwind_params(DataContainer()))
        pb.AddInitial(InitialTimeFixed(), DataContainer().double(0.0))
        pb.AddInitial(InitialSpaceFixed(), DataContainer().vec((0.1 * ONE_AU, 0, 0)))
        pb.AddInitial(InitialMomentumShell(), DataContainer().double(p0))
        pb.AddDiffusion(DiffusionIsotropicConstant(), DataContainer().double(d0))
        pb.AddBoundary(BoundaryTimeExpire(), _boundary(DataContainer(), 1, [-1]).double(t_max))
        pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [-1]).vec((0, 0, 0)).double(0.05 * ONE_AU))
        pb.AddBoundary(BoundarySphereAbsorb(), _boundary(DataContainer(), 1, [-1]).vec((0, 0, 0)).double(5.0 * ONE_AU))
        pb.AddBoundary(BoundarySpherePass(), _boundary(DataContainer(), -1, [0]).vec((0, 0, 0)).double(ONE_AU))
        c = distro_header(DataContainer(), (n_t, n_mu, 0), (0.0, -1.0, 0.0), (t_max, 1.0, 1.0),
                          unit_val=(U.unit_time, 1.0, 1.0))
        c.double(1.0).double(0.0)
        pb.AddDistribution(DistributionTimeMu(), c)
        pb.options[SPX_OPT_PA_SCATTERING] = 1.0
        out.append(pb)
    return out


# option numbers (include/spx.h)
SPX_OPT_STEPS_PER_ORBIT = 1
SPX_OPT_DERIV_MODE = 2
SPX_OPT_PA_SCATTERING = 3
SPX_OPT_RECORD_FINAL = 4
SPX_OPT_MU_METHOD = 8
SPX_OPT_PERP_METHOD = 9
