"""Plugin prototypes with the reference's class names.

In the reference a user passes a default-constructed plugin object plus a ``DataContainer`` to
``Add*`` (src/simulation.hh:93-138; e.g. ``AddBackground(BackgroundUniform(), container)``). The
objects here play the same role: an instance only names the class; its parameters come from the
container. Each class carries the role and the kind number that ``spx_add_plugin`` takes
(include/spx.h lists the same numbers).

Classes marked "extension" have no counterpart in the reference; they exist because a workload
needs a sampler, boundary or histogram the reference does not provide.
"""
from __future__ import annotations

ROLE_BACKGROUND = 0
ROLE_DIFFUSION = 1
ROLE_SOURCE = 2
ROLE_BOUNDARY = 3
ROLE_INITIAL = 4
ROLE_DISTRIBUTION = 5

ROLE_NAMES = {ROLE_BACKGROUND: "background", ROLE_DIFFUSION: "diffusion", ROLE_SOURCE: "source",
              ROLE_BOUNDARY: "boundary", ROLE_INITIAL: "initial", ROLE_DISTRIBUTION: "distribution"}


class Plugin:
    role: int = -1
    kind: int = -1
    #: the reference class this mirrors (None for an extension)
    reference: str | None = None

    @property
    def name(self) -> str:
        return type(self).__name__

    def __repr__(self) -> str:
        return f"{self.name}()"


_REGISTRY: dict[tuple[int, int], type] = {}


def _plugin(role: int, kind: int, reference: bool = True):
    def deco(cls):
        cls.role = role
        cls.kind = kind
        cls.reference = cls.__name__ if reference else None
        _REGISTRY[(role, kind)] = cls
        return cls
    return deco


def by_kind(role: int, kind: int) -> type:
    return _REGISTRY[(role, kind)]


def all_plugins() -> list[type]:
    return list(_REGISTRY.values())


# -- backgrounds (src/background_*.hh) ---------------------------------------------------------
@_plugin(ROLE_BACKGROUND, 1)
class BackgroundUniform(Plugin): pass  # src/background_uniform.cc:49-88


@_plugin(ROLE_BACKGROUND, 2)
class BackgroundShock(Plugin): pass  # src/background_shock.cc:58-128


@_plugin(ROLE_BACKGROUND, 3)
class BackgroundSmoothShock(Plugin): pass  # src/background_smooth_shock.cc:46-197


@_plugin(ROLE_BACKGROUND, 4)
class BackgroundDipole(Plugin): pass  # src/background_dipole.cc:48-125


@_plugin(ROLE_BACKGROUND, 5)
class BackgroundSolarWind(Plugin): pass  # src/background_solarwind.cc:58-314


@_plugin(ROLE_BACKGROUND, 7)
class BackgroundDiscontinuity(Plugin): pass  # src/background_discontinuity.cc:51-104 (runs on the shock kernels)


@_plugin(ROLE_BACKGROUND, 8)
class BackgroundSmoothDiscontinuity(Plugin): pass  # src/background_smooth_discontinuity.cc:46-178 (smooth-shock kernels)


@_plugin(ROLE_BACKGROUND, 6)
class BackgroundServerCartesian(Plugin):
    """The base parameters only (src/background_base.cc:342-346); the grid itself comes with
    Problem.grid / spx_set_background_grid (src/background_server_cartesian.cc, first-order
    interpolation of src/server_cartesian.cc:206-840 on one block)."""


# -- diffusion (src/diffusion_other.hh) --------------------------------------------------------
@_plugin(ROLE_DIFFUSION, 1)
class DiffusionIsotropicConstant(Plugin): pass  # src/diffusion_other.cc:64-79


@_plugin(ROLE_DIFFUSION, 2)
class DiffusionQLTConstant(Plugin): pass  # src/diffusion_other.cc:145-149


@_plugin(ROLE_DIFFUSION, 3)
class DiffusionParaConstant(Plugin): pass  # src/diffusion_other.cc:381-408


@_plugin(ROLE_DIFFUSION, 4)
class DiffusionPerpConstant(Plugin): pass  # src/diffusion_other.cc:459-486


@_plugin(ROLE_DIFFUSION, 5)
class DiffusionFullConstant(Plugin): pass  # src/diffusion_other.cc:538-566


@_plugin(ROLE_DIFFUSION, 6)
class DiffusionFlowMomentumPowerLaw(Plugin): pass  # src/diffusion_other.cc:622-653


@_plugin(ROLE_DIFFUSION, 7)
class DiffusionKineticEnergyRadialDistancePowerLaw(Plugin): pass  # src/diffusion_other.cc:713-752


@_plugin(ROLE_DIFFUSION, 8)
class DiffusionRigidityMagneticFieldPowerLaw(Plugin): pass  # src/diffusion_other.cc:804-833


@_plugin(ROLE_DIFFUSION, 9)
class DiffusionStraussEtAl2013(Plugin): pass  # src/diffusion_other.cc:886-914


@_plugin(ROLE_DIFFUSION, 10)
class DiffusionPotgieterEtAl2015(Plugin): pass  # src/diffusion_other.cc:968-996


@_plugin(ROLE_DIFFUSION, 11)
class DiffusionEmpiricalSOQLTandUNLT(Plugin): pass  # src/diffusion_other.cc:1049-1082


@_plugin(ROLE_DIFFUSION, 12)
class DiffusionWNLTConstant(Plugin):
    """A2A, l_max, ps_index (as QLT), A2T, A2L (src/diffusion_other.cc:202-243): K_perp from the weakly nonlinear
    model and the QLT pitch-angle coefficient (USE_QLT_SCATT_WITH_WNLT_DIFF, src/diffusion_other.hh:137)."""


@_plugin(ROLE_DIFFUSION, 13)
class DiffusionWNLTRampVLISM(Plugin):
    """The WNLT parameters, then l_max_HP, z_nose, z_sheath (src/diffusion_other.cc:281-327): the largest
    turbulent scale ramps linearly across the heliosheath between two Rankine half bodies."""


# -- sources (src/source_other.hh) -------------------------------------------------------------
@_plugin(ROLE_SOURCE, 1)
class SourceConstant(Plugin): pass


@_plugin(ROLE_SOURCE, 2)
class SourceMomentumInjection(Plugin): pass  # src/source_other.cc:113-118


@_plugin(ROLE_SOURCE, 3)
class SourceSphericalShockInjection(Plugin): pass  # src/source_other.cc:150-177 (p_inj, r0, r_sh, w_sh, rate)


# -- boundaries (src/boundary_*.hh) ------------------------------------------------------------
@_plugin(ROLE_BOUNDARY, 1)
class BoundaryTimeExpire(Plugin): pass  # src/boundary_time.cc:70-118


@_plugin(ROLE_BOUNDARY, 2)
class BoundaryTimePass(Plugin): pass  # src/boundary_time.cc:126-160


@_plugin(ROLE_BOUNDARY, 3)
class BoundaryTimeRecurrent(Plugin): pass  # src/boundary_time.cc:168-208


@_plugin(ROLE_BOUNDARY, 10)
class BoundaryPlaneAbsorb(Plugin): pass  # src/boundary_space.cc:71-126


@_plugin(ROLE_BOUNDARY, 11)
class BoundaryPlaneReflect(Plugin): pass  # src/boundary_space.cc:136-165


@_plugin(ROLE_BOUNDARY, 12)
class BoundaryPlanePass(Plugin): pass  # src/boundary_space.cc:175-203


@_plugin(ROLE_BOUNDARY, 13)
class BoundaryBoxReflect(Plugin): pass  # src/boundary_space.cc:249-337


@_plugin(ROLE_BOUNDARY, 14)
class BoundarySphereAbsorb(Plugin): pass  # src/boundary_space.cc:395-454


@_plugin(ROLE_BOUNDARY, 15)
class BoundarySphereReflect(Plugin): pass  # src/boundary_space.cc:464-493


@_plugin(ROLE_BOUNDARY, 16)
class BoundaryRankineAbsorb(Plugin): pass  # src/boundary_space.cc:552-601


@_plugin(ROLE_BOUNDARY, 17)
class BoundaryCylinderAbsorb(Plugin): pass  # src/boundary_space.cc:647-729


@_plugin(ROLE_BOUNDARY, 18)
class BoundaryRegionAbsorb(Plugin): pass  # src/boundary_space.cc:775-848


@_plugin(ROLE_BOUNDARY, 19, reference=False)
class BoundarySpherePass(Plugin):
    """Extension: an event sphere that records every crossing and never stops the trajectory.

    Parameters follow BoundarySphere (int max_crossings, ints actions, GeoVector origin, double
    radius); max_crossings < 0 means unlimited, max_crossings == 1 makes it terminal, exactly as
    for BoundaryPlanePass (src/boundary_space.cc:198-203)."""


@_plugin(ROLE_BOUNDARY, 30)
class BoundaryMomentumInject(Plugin): pass  # src/boundary_momentum.cc:69-130


@_plugin(ROLE_BOUNDARY, 31)
class BoundaryMomentumPass(Plugin): pass  # src/boundary_momentum.cc:140-168


@_plugin(ROLE_BOUNDARY, 32)
class BoundaryMomentumInjectRestrictSlab(Plugin): pass  # src/boundary_momentum.cc:201-223


@_plugin(ROLE_BOUNDARY, 33)
class BoundaryMomentumInjectRestrictShell(Plugin): pass  # src/boundary_momentum.cc:256-278


@_plugin(ROLE_BOUNDARY, 34)
class BoundaryMirror(Plugin): pass  # src/boundary_momentum.cc:329-339


# -- initial conditions (src/initial_*.hh) -----------------------------------------------------
@_plugin(ROLE_INITIAL, 1)
class InitialTimeFixed(Plugin): pass  # src/initial_time.cc:48-65


@_plugin(ROLE_INITIAL, 2)
class InitialTimeInterval(Plugin): pass  # src/initial_time.cc:114-140


@_plugin(ROLE_INITIAL, 10)
class InitialSpaceFixed(Plugin): pass  # src/initial_space.cc:49-66


@_plugin(ROLE_INITIAL, 11)
class InitialSpaceLine(Plugin): pass  # src/initial_space.cc:115-141


@_plugin(ROLE_INITIAL, 12)
class InitialSpaceCircle(Plugin): pass  # src/initial_space.cc:190-214


@_plugin(ROLE_INITIAL, 13)
class InitialSpaceBox(Plugin): pass  # src/initial_space.cc:248-251


@_plugin(ROLE_INITIAL, 14)
class InitialSpaceSphere(Plugin): pass  # src/initial_space.cc:297-319


@_plugin(ROLE_INITIAL, 15)
class InitialSpaceSphereSector(Plugin): pass  # src/initial_space.cc:357-394


@_plugin(ROLE_INITIAL, 16)
class InitialSpaceRankineHalfBody(Plugin): pass  # src/initial_space.cc:432-463


@_plugin(ROLE_INITIAL, 17)
class InitialSpaceCylinder(Plugin): pass  # src/initial_space.cc:561-583 (origin, height, radius vector)


@_plugin(ROLE_INITIAL, 18)
class InitialSpaceCylinderSector(Plugin): pass  # src/initial_space.cc:621-645 (... and phi1, phi2)


@_plugin(ROLE_INITIAL, 30)
class InitialMomentumFixed(Plugin): pass  # src/initial_momentum.cc:51-98


@_plugin(ROLE_INITIAL, 31)
class InitialMomentumBeam(Plugin): pass  # src/initial_momentum.cc:139-162


@_plugin(ROLE_INITIAL, 32)
class InitialMomentumRing(Plugin): pass  # src/initial_momentum.cc:203-244


@_plugin(ROLE_INITIAL, 33)
class InitialMomentumShell(Plugin): pass  # src/initial_momentum.cc:283-326


@_plugin(ROLE_INITIAL, 34)
class InitialMomentumThickShell(Plugin): pass  # src/initial_momentum.cc:363-412


@_plugin(ROLE_INITIAL, 35)
class InitialMomentumMaxwell(Plugin): pass  # src/initial_momentum.cc:503-555


@_plugin(ROLE_INITIAL, 40, reference=False)
class InitialMomentumLogEnergyPitchBand(Plugin):
    """Extension: kinetic energy log-uniform in [E1, E2], pitch-angle cosine uniform in
    [mu1, mu2] about the local field, gyrophase uniform (Lorentz; Focused uses (p, mu)).

    Parameters: double E1, double E2, double mu1, double mu2 (code units of energy). The
    reference has no sampler that is log-uniform in energy or limits the pitch angle; its nearest
    are InitialMomentumThickShell (log-uniform in momentum, src/initial_momentum.cc:381-412) and
    InitialMomentumRing (fixed pitch, src/initial_momentum.cc:226-244)."""


@_plugin(ROLE_INITIAL, 41, reference=False)
class InitialSpaceEquatorialBand(Plugin):
    """Extension: a point on the equator of a dipole at radius L*r_ref, L uniform in [L1, L2],
    azimuth uniform. Parameters: GeoVector origin, double r_ref, double L1, double L2."""


# -- distributions (src/distribution_other.hh) -------------------------------------------------
@_plugin(ROLE_DISTRIBUTION, 1)
class DistributionTimeUniform(Plugin): pass  # src/distribution_other.cc


@_plugin(ROLE_DISTRIBUTION, 2)
class DistributionPositionUniform(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 3)
class DistributionMomentumUniform(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 4)
class DistributionPositionMomentumUniform(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 5)
class DistributionSpectrumKineticEnergyPowerLaw(Plugin): pass  # src/distribution_other.cc:520-602


@_plugin(ROLE_DISTRIBUTION, 6)
class DistributionSpectrumKineticEnergyBentPowerLaw(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 7)
class DistributionPositionCumulativeOrder1(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 8)
class DistributionPositionCumulativeOrder2(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 9)
class DistributionDivergenceFlowPowerLaw(Plugin): pass


@_plugin(ROLE_DISTRIBUTION, 10)
class DistributionLossCone(Plugin):
    """src/distribution_other.cc:794-862: the first or the final position (val_time), Cartesian or
    spherical (val_coord), weighted by (|B|_min, |B|_max, asin(sqrt(|B| / |B|_max))) along the
    trajectory. The extrema are tracked whenever a problem has this distribution, as a reference
    build with RECORD_BMAG_EXTREMA does (src/trajectory_base.hh:31). All three dimensions binned."""


@_plugin(ROLE_DISTRIBUTION, 11)
class DistributionAnisotropyLISM(Plugin):
    """src/distribution_other.cc:364-483 (Lorentz trajectories only): the first point's momentum
    direction in a given frame, binned in (theta, phi); weights: Compton-Getting factor, momentum
    power-law, first and second Legendre anisotropy of the LISM-frame momentum against the field, and
    the guiding centre dotted with a density gradient. Parameters: the DistributionTemplated header,
    GeoVector rot_matrix[3], GeoVector U_LISM, double mom_pow_law, GeoVector grad_perp_dens. The
    reference's set-up accepts bins in the first and third dimensions only (dims 5) while it sets the
    first two values; the third value is 0 here (unset there)."""


@_plugin(ROLE_DISTRIBUTION, 20, reference=False)
class DistributionTimeMu(Plugin):
    """Extension: a (t, mu) histogram of the second point (the event), for observer crossings
    in focused transport. Parameters: the DistributionTemplated header (n_bins, minval, maxval,
    log_bins, bin_outside, unit_distro, unit_val, keep_records) and double val_hot, double
    val_cold, as DistributionUniform (src/distribution_other.cc:30-60)."""


#: number of doubles per bin of a distribution kind (DistributionTemplated<double|GeoVector|GeoMatrix>)
DISTRO_WIDTH = {1: 1, 2: 1, 3: 1, 4: 1, 5: 1, 6: 1, 7: 3, 8: 9, 9: 1, 10: 3, 20: 1}
