"""Unit system and proton kinematics of the reference, for building plugin parameters on the host.

The reference works in code units fixed at compile time (common/specie.hh:30-82): length
1e10 cm, velocity 0.1 c, mass m_p, charge e; time, field, momentum, energy and diffusion units
derive from those. The particle is a proton (common/params.hh:107). The physical constants are
the reference's own values (common/physical_constants.hh:20-81).
"""
from __future__ import annotations

import math

SPEED_OF_LIGHT = 2.99792458e10          # cm/s
MASS_PROTON = 1.67262192596e-24         # g
ELECTRON_CHARGE = 4.8032044e-10         # Fr
ELECTRON_VOLT = 1.602176634e-12         # erg
MEV = 1.0e6 * ELECTRON_VOLT
GEV = 1.0e9 * ELECTRON_VOLT
ASTRONOMICAL_UNIT = 1.495978707e13      # cm

unit_length = 1.0e10
unit_velocity = 0.1 * SPEED_OF_LIGHT
unit_mass = MASS_PROTON
unit_charge = ELECTRON_CHARGE
unit_momentum = unit_mass * unit_velocity
unit_energy = unit_mass * unit_velocity * unit_velocity
unit_time = unit_length / unit_velocity
unit_magnetic = unit_momentum / (unit_charge * unit_time)
unit_diffusion = unit_velocity * unit_length
c_code = SPEED_OF_LIGHT / unit_velocity

# proton in code units
mass = 1.0
charge = 1.0


def EnrTot(p: float) -> float:  # noqa: N802 (reference name, common/physics.hh:288)
    return math.sqrt(p * p + (mass * c_code) ** 2) * c_code


def EnrKin(p: float) -> float:  # noqa: N802 (common/physics.hh:302)
    return EnrTot(p) - mass * c_code * c_code


def Mom(enr_kin: float) -> float:  # noqa: N802 (common/physics.hh:274)
    return math.sqrt(enr_kin * (enr_kin + 2.0 * mass * c_code * c_code)) / c_code


def Vel(p: float) -> float:  # noqa: N802 (common/physics.hh:316)
    return p * c_code * c_code / EnrTot(p)


def Rigidity(p: float) -> float:  # noqa: N802 (common/physics.hh:363)
    return p * c_code / abs(charge)


def LarmorRadius(p: float, bmag: float) -> float:  # noqa: N802 (common/physics.hh:453)
    return p * c_code / (abs(charge) * bmag)


def CyclotronFrequency(v: float, bmag: float) -> float:  # noqa: N802 (common/physics.hh:438)
    gamma = 1.0 / math.sqrt(1.0 - (v / c_code) ** 2)
    return charge * bmag / (gamma * mass * c_code)


def mev_to_mom(e_mev: float) -> float:
    """Code-unit momentum of a proton with kinetic energy ``e_mev`` MeV."""
    return Mom(e_mev * MEV / unit_energy)
