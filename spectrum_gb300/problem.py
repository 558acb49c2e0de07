"""A simulation problem: configure-time physics choices plus a list of set-up plugins.

The reference fixes the trajectory type, time flow and Runge-Kutta table at configure time
(configure.ac:236-295) and receives every plugin as ``Add*(Prototype(), DataContainer)``. A
``Problem`` records the same information in a form that can be handed to the C ABI
(``spx_create`` + ``spx_add_plugin``) or serialised for the reference's own code (the oracle
harness reads the byte format written by ``to_spec``).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

from . import plugins as P
from .datacontainer import DataContainer

# trajectory types: the reference's configure.ac:236-244 numbering
TRAJ_FIELDLINE = 199
TRAJ_LORENTZ = 200
TRAJ_GUIDING = 201
TRAJ_GUIDING_SCATT = 202
TRAJ_GUIDING_DIFF = 203
TRAJ_GUIDING_DIFF_SCATT = 204
TRAJ_FOCUSED = 205
TRAJ_PARKER = 206
TRAJ_PARKER_SOURCE = 207
TRAJ_NAMES = {TRAJ_FIELDLINE: "TrajectoryFieldline", TRAJ_LORENTZ: "TrajectoryLorentz", TRAJ_GUIDING: "TrajectoryGuiding",
              TRAJ_GUIDING_SCATT: "TrajectoryGuidingScatt", TRAJ_GUIDING_DIFF: "TrajectoryGuidingDiff",
              TRAJ_GUIDING_DIFF_SCATT: "TrajectoryGuidingDiffScatt", TRAJ_FOCUSED: "TrajectoryFocused",
              TRAJ_PARKER: "TrajectoryParker", TRAJ_PARKER_SOURCE: "TrajectoryParkerSource"}

FORWARD = 0
BACKWARD = 1


@dataclass
class PluginEntry:
    plugin: P.Plugin
    blob: bytes
    n_records: int


@dataclass
class Grid:
    """One uniform Cartesian block: node (i, j, k) at cent_min + (i, j, k) * zone_length; values
    of shape (n[2], n[1], n[0], 6) holding U then B at each node (code units)."""
    n: tuple
    cent_min: tuple
    zone_length: tuple
    values: "object"

    @classmethod
    def sample(cls, n, cent_min, zone_length, fields) -> "Grid":
        """Sample fields(x, y, z) -> (U, B) (arrays of shape (..., 3)) at the nodes."""
        import numpy as np
        ax = [cent_min[k] + zone_length[k] * np.arange(n[k]) for k in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        u, b = fields(x, y, z)
        values = np.concatenate([u, b], axis=-1).astype(np.float64)
        return cls(tuple(int(v) for v in n), tuple(float(v) for v in cent_min), tuple(float(v) for v in zone_length),
                   np.ascontiguousarray(values))


@dataclass
class BlockGrid:
    """The data of the reference's Cartesian data server (its reader's files, src/reader_cartesian.cc):
    n_blocks blocks of 4^3 zones per axis spanning [domain_min, domain_max] (au); values of shape
    (blocks, 64, 6) -- blocks x fastest, in each block zones x fastest -- holding U then B in the
    reference's fluid units; ghost_cells ghost layers per block side (SERVER_NUM_GHOST_CELLS)."""
    n_blocks: tuple
    domain_min: tuple
    domain_max: tuple
    values: "object"
    ghost_cells: int = 0
    #: SERVER_INTERP_ORDER: 1 the 8-zone stencil, 0 the zone's values, -1 the reader's interpolation
    interp_order: int = 1

    @classmethod
    def read(cls, dat_path: str, ghost_cells: int = 0) -> "BlockGrid":
        """The reader's pair of files: the binary block data ``name.dat`` (the server reads
        ``<pattern>.out``) and its text header ``name.info``, the data file's name with its last four
        characters replaced (blocks per axis, domain minimum, domain maximum, variables per zone)."""
        import numpy as np
        with open(dat_path[:-4] + ".info") as f:
            tok = f.read().split()
        nb = tuple(int(x) for x in tok[0:3])
        dmin = tuple(float(x) for x in tok[3:6])
        dmax = tuple(float(x) for x in tok[6:9])
        nvar = int(tok[9])
        if nvar != 6:
            raise ValueError("the Cartesian server reads six variables per zone (U, B)")
        values = np.fromfile(dat_path, dtype="<f8", count=nb[0] * nb[1] * nb[2] * 64 * nvar)
        return cls(nb, dmin, dmax, values.reshape(-1, 64, nvar), ghost_cells)

    def write(self, dat_path: str) -> None:
        """Write the reader's two files (name.dat and name.info)."""
        import numpy as np
        with open(dat_path[:-4] + ".info", "w") as f:
            f.write("%d %d %d\n%r %r %r\n%r %r %r\n6\n" % (*self.n_blocks, *self.domain_min, *self.domain_max))
        np.ascontiguousarray(self.values, dtype="<f8").tofile(dat_path)

    @classmethod
    def sample(cls, n_blocks, domain_min, domain_max, fields, ghost_cells: int = 0) -> "BlockGrid":
        """Sample fields(x, y, z) -> (U, B) (arrays of shape (..., 3), fluid units, x in au) at the zone
        centres of every block."""
        import numpy as np
        nb = [int(v) for v in n_blocks]
        zl = [(domain_max[k] - domain_min[k]) / nb[k] / 4.0 for k in range(3)]
        ax = [domain_min[k] + zl[k] * (np.arange(4 * nb[k]) + 0.5) for k in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        u, b = fields(x, y, z)
        glob = np.concatenate([u, b], axis=-1).astype(np.float64)  # (4 nz, 4 ny, 4 nx, 6)
        blk = glob.reshape(nb[2], 4, nb[1], 4, nb[0], 4, 6).transpose(0, 2, 4, 1, 3, 5, 6)
        return cls(tuple(nb), tuple(float(v) for v in domain_min), tuple(float(v) for v in domain_max),
                   np.ascontiguousarray(blk.reshape(-1, 64, 6)), int(ghost_cells))


@dataclass
class Problem:
    traj: int = TRAJ_PARKER
    time_flow: int = FORWARD
    rk: int = 0
    plugins: list[PluginEntry] = field(default_factory=list)
    seed: int = 0x5EED0000
    n_traj: int = 1000
    problem_id: int = 0
    #: options of the stepping kernel (see include/spx.h, SPX_OPT_*)
    options: dict[int, float] = field(default_factory=dict)
    #: the data of a gridded background (BackgroundServerCartesian): a Grid (one uniform block in code
    #: units), a BlockGrid (the reference server's blocks), or None
    grid: "Grid | BlockGrid | None" = None

    def add(self, plugin: P.Plugin, container: DataContainer) -> "Problem":
        self.plugins.append(PluginEntry(plugin, container.data(), container.size()))
        return self

    # reference-style method names
    def AddBackground(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_BACKGROUND, proto, c)

    def AddDiffusion(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_DIFFUSION, proto, c)

    def AddSource(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_SOURCE, proto, c)

    def AddBoundary(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_BOUNDARY, proto, c)

    def AddInitial(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_INITIAL, proto, c)

    def AddDistribution(self, proto, c):  # noqa: N802
        return self._add_role(P.ROLE_DISTRIBUTION, proto, c)

    def _add_role(self, role, proto, c):
        if proto.role != role:
            raise TypeError(f"{proto.name} is not a {P.ROLE_NAMES[role]} plugin")
        return self.add(proto, c)

    def replace(self, role: int, slot: int, plugin: P.Plugin, container: DataContainer) -> "Problem":
        """Replace the ``slot``-th plugin of ``role`` (used to derive batched problems)."""
        idx = [i for i, e in enumerate(self.plugins) if e.plugin.role == role]
        self.plugins[idx[slot]] = PluginEntry(plugin, container.data(), container.size())
        return self

    def distributions(self) -> list[PluginEntry]:
        return [e for e in self.plugins if e.plugin.role == P.ROLE_DISTRIBUTION]

    def normals_per_step(self) -> int:
        """Normal draws per step of the trajectory type (3 for Parker: src/trajectory_parker.cc:159-180;
        1 for GuidingScatt, whose k-th normal, redraws included, is the first of block k)."""
        if self.traj in (TRAJ_PARKER, TRAJ_PARKER_SOURCE):
            return 3
        return 1

    def to_spec(self, max_attempts: int = 100) -> bytes:
        """Serialise for the oracle harness (format documented in oracle/ref_glue/harness.cc)."""
        out = bytearray(b"SPXS")
        out += struct.pack("<IQIIIII", 1, self.seed, self.n_traj, self.problem_id,
                           self.normals_per_step(), max_attempts, len(self.plugins))
        for e in self.plugins:
            name = e.plugin.name.encode()
            out += struct.pack("<II", e.plugin.role, len(name)) + name
            out += struct.pack("<II", e.n_records, len(e.blob)) + e.blob
        return bytes(out)


def distro_header(c: DataContainer, n_bins, minval, maxval, log_bins=(0, 0, 0), bin_outside=(0, 0, 0),
                  unit_distro=1.0, unit_val=(1.0, 1.0, 1.0), keep_records=False, width=1) -> DataContainer:
    """The DistributionTemplated part of a distribution container (src/distribution_templated.cc:92-108)."""
    c.mi(n_bins).vec(minval).vec(maxval).mi(log_bins).mi(bin_outside)
    if width == 1:
        c.double(unit_distro)
    elif width == 3:
        c.vec(unit_distro if hasattr(unit_distro, "__len__") else (unit_distro,) * 3)
    else:
        c.mat([[unit_distro] * 3] * 3)
    c.vec(unit_val).bool(keep_records)
    return c
