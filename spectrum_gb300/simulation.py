"""SimulationGPU: the reference's simulation interface on top of the C ABI.

The method names and argument meanings are those of SimulationWorker (src/simulation.hh:93-138):
Add{Background,Diffusion,Source,Boundary,Initial,Distribution}(prototype, container), SetTasks,
MainLoop, PrintDistro1D, PrintDistro2D, PrintRecords, RestoreDistro, DistroFileName, GetTrajectoryName. Instead of an MPI farm
the trajectories run in one device launch; SetTasks may be called several times to batch many
problems, each optionally replacing plugins of the base set (``AddProblem``).

``run_problems`` runs a list of ``Problem`` objects (spectrum_gb300.problem) that share their
plugin structure as one batched launch.
"""
from __future__ import annotations

import struct

import numpy as np

from . import capi, distro_print
from . import plugins as P
from .datacontainer import DataContainer
from .problem import TRAJ_NAMES, Problem
from .workloads import SPX_OPT_DERIV_MODE, SPX_OPT_PA_SCATTERING, SPX_OPT_RECORD_FINAL, SPX_OPT_STEPS_PER_ORBIT


class SimulationGPU:
    def __init__(self, traj: int, time_flow: int = 0, rk: int = 0, precision: int = capi.SPX_FP64,
                 options: dict[int, float] | None = None):
        self.traj = traj
        self.ctx = capi.Context(traj, time_flow, rk, precision)
        self.precision = precision
        for k, v in (options or {}).items():
            self.ctx.set_option(k, v)
        self._distro_names: list[str] = []
        # each distribution's parameter container, and per problem the ones AddProblem replaced (the
        # text output reads the binning from them)
        self._distro_blobs: list[bytes] = []
        self._problem_distro_blobs: list[dict[int, bytes]] = []
        self._file_prefix = ""
        self._restore: set[int] = set()
        self._n_problems = 0
        self.stats: capi.Stats | None = None

    # -- plugin set-up (src/simulation.hh:105-123) ----------------------------------------------
    def _add(self, role: int, proto: P.Plugin, container: DataContainer) -> None:
        if proto.role != role:
            raise TypeError(f"{proto.name} is not a {P.ROLE_NAMES[role]} plugin")
        self.ctx.add_plugin(role, proto.kind, container.data(), container.size())
        if role == P.ROLE_DISTRIBUTION:
            self._distro_names.append(proto.name)
            self._distro_blobs.append(container.data())

    def AddBackground(self, proto, container, fname_pattern_in: str = "", ghost_cells: int = 0):  # noqa: N802
        """With a file-name pattern, a BackgroundServerCartesian reads its data as the reference's server
        does: the reader's blocks from <pattern>.out and their header from <pattern>.info
        (ServerCartesianBack::ServerStart, src/server_cartesian.cc:931-933, and ReadCartesianHeader,
        src/reader_cartesian.cc:36). ``ghost_cells`` stands for the build's SERVER_NUM_GHOST_CELLS."""
        self._add(P.ROLE_BACKGROUND, proto, container)
        if fname_pattern_in and proto.name == "BackgroundServerCartesian":
            from .problem import BlockGrid
            g = BlockGrid.read(fname_pattern_in + ".out", ghost_cells)
            self.ctx.set_background_blocks(g.n_blocks, g.domain_min, g.domain_max, g.ghost_cells, g.values)

    def SetBackgroundGrid(self, grid) -> None:  # noqa: N802
        """The block of a BackgroundServerCartesian background (a problem.Grid); takes the place of
        the data files the reference's server reads."""
        self.ctx.set_background_grid(grid.n, grid.cent_min, grid.zone_length, grid.values)

    def AddDiffusion(self, proto, container):  # noqa: N802
        self._add(P.ROLE_DIFFUSION, proto, container)

    def AddSource(self, proto, container):  # noqa: N802
        self._add(P.ROLE_SOURCE, proto, container)

    def AddBoundary(self, proto, container):  # noqa: N802
        self._add(P.ROLE_BOUNDARY, proto, container)

    def AddInitial(self, proto, container):  # noqa: N802
        self._add(P.ROLE_INITIAL, proto, container)

    def AddDistribution(self, proto, container):  # noqa: N802
        self._add(P.ROLE_DISTRIBUTION, proto, container)

    # -- tasks and the main loop -----------------------------------------------------------------
    def SetTasks(self, n_traj: int, batch_size: int = 0, max_traj_per_worker: int = 0, seed: int = 0x5EED0000):  # noqa: N802
        """One problem of n_traj trajectories (batch sizes belong to the MPI farm and are ignored)."""
        self.ctx.add_problem(n_traj, seed)
        self._n_problems += 1
        self._problem_distro_blobs.append({})

    def AddProblem(self, n_traj: int, seed: int, overrides=()):  # noqa: N802
        """A further problem: ``overrides`` is a list of (role, slot, prototype, DataContainer)."""
        blob = bytearray()
        replaced = {}
        for role, slot, proto, c in overrides:
            data = c.data()
            blob += struct.pack("<5I", role, slot, proto.kind, c.size(), len(data)) + data
            if role == P.ROLE_DISTRIBUTION:
                replaced[slot] = data
        self.ctx.add_problem(n_traj, seed, bytes(blob))
        self._n_problems += 1
        self._problem_distro_blobs.append(replaced)

    def MainLoop(self, tuning: capi.Tuning | None = None) -> capi.Stats:  # noqa: N802
        """Restore the distributions flagged by RestoreDistro, run every problem's trajectories, and,
        when DistroFileName gave a file name, dump every distribution (src/simulation.cc:705-793).
        Distributions accumulate over MainLoop calls (reset them with ctx.reset_distributions)."""
        for d in sorted(self._restore):
            for p in range(self._n_problems):
                try:
                    self.ctx.restore_distribution(p, d, self.distro_path(d, p))
                except capi.SpxError as e:
                    # DistributionTemplated::Restore returns quietly on a missing file or another class
                    if e.code not in (capi.SPX_ERR_IO, capi.SPX_ERR_MISMATCH):
                        raise
        self.ctx.run(tuning)
        self.stats = self.ctx.sync()
        if self._file_prefix:
            self.DumpDistro()
        return self.stats

    def GetTrajectoryName(self) -> str:  # noqa: N802
        return TRAJ_NAMES.get(self.traj, "Trajectory")

    def DistroFileName(self, file_name: str) -> None:  # noqa: N802
        """Prefix of the dump files: distribution d of the first problem is <prefix><d>.out, the
        reference's name (src/simulation.cc:790-793); of problem p > 0, <prefix><d>_problem<p>.out."""
        self._file_prefix = file_name

    def distro_path(self, distro: int, problem: int = 0) -> str:
        suffix = "" if problem == 0 else f"_problem{problem}"
        return f"{self._file_prefix}{distro}{suffix}.out"

    def RestoreDistro(self, distro: int) -> None:  # noqa: N802
        """Flag distribution ``distro`` to be restored from its dump file when MainLoop starts
        (SimulationMaster::RestoreDistro, src/simulation.cc:714-720)."""
        self._restore.add(distro)

    def DumpDistro(self) -> None:  # noqa: N802
        """Every distribution of every problem in the reference's dump-file layout."""
        for p in range(self._n_problems):
            for d in range(len(self._distro_names)):
                self.ctx.dump_distribution(p, d, self.distro_path(d, p))

    def distribution(self, distro: int, problem: int = 0):
        return self.ctx.distribution(problem, distro)

    def _distro_header(self, distro: int, problem: int) -> distro_print.DistroHeader:
        blob = self._problem_distro_blobs[problem].get(distro, self._distro_blobs[distro]) \
            if problem < len(self._problem_distro_blobs) else self._distro_blobs[distro]
        _, width = self.ctx.distribution_info(problem, distro)
        return distro_print.DistroHeader.from_container(blob, width)

    def PrintDistro1D(self, distro: int, ijk: int, file_name: str, phys_units: bool = False, problem: int = 0) -> None:  # noqa: N802
        """The distribution along axis ``ijk``, the other two collapsed, in the text layout of
        DistributionTemplated::Print1D (SimulationMaster::PrintDistro1D, src/simulation.cc:856-859)."""
        counts, sums, n_events = self.distribution(distro, problem)
        distro_print.print_1d(file_name, self._distro_header(distro, problem), counts, sums, n_events, ijk, phys_units)

    def PrintDistro2D(self, distro: int, ijk1: int, ijk2: int, file_name: str, phys_units: bool = False,  # noqa: N802
                      problem: int = 0) -> None:
        """The distribution over axes ``ijk1`` and ``ijk2``, the third collapsed, in the text layout of
        DistributionTemplated::Print2D (SimulationMaster::PrintDistro2D, src/simulation.cc:871-874)."""
        counts, sums, n_events = self.distribution(distro, problem)
        distro_print.print_2d(file_name, self._distro_header(distro, problem), counts, sums, n_events, ijk1, ijk2,
                              phys_units)

    def PrintRecords(self, distro: int, file_name: str, phys_units: bool = False, problem: int = 0) -> None:  # noqa: N802
        """The records of a distribution that keeps them, in the text layout of
        DistributionTemplated::PrintRecords (SimulationMaster::PrintRecords, src/simulation.cc:883-886).
        The device appends records in completion order; the reference in trajectory order."""
        values, weights, _ = self.ctx.distribution_records(problem, distro)
        distro_print.print_records(file_name, self._distro_header(distro, problem), values, weights, phys_units)

    def close(self) -> None:
        self.ctx.close()


def _diff_overrides(base: Problem, other: Problem) -> bytes:
    if [(e.plugin.role, e.plugin.kind) for e in base.plugins] != [(e.plugin.role, e.plugin.kind) for e in other.plugins]:
        raise ValueError("batched problems must share their plugin structure")
    out = bytearray()
    slots: dict[int, int] = {}
    for eb, eo in zip(base.plugins, other.plugins):
        role = eb.plugin.role
        slot = slots.get(role, 0)
        slots[role] = slot + 1
        if eb.blob != eo.blob:
            if role == P.ROLE_BOUNDARY:
                raise ValueError("boundaries of batched problems must agree (replace them by slot via AddProblem)")
            out += struct.pack("<5I", role, slot, eo.plugin.kind, eo.n_records, len(eo.blob)) + eo.blob
    return bytes(out)


def open_problems(problems: list[Problem] | Problem, precision: int = capi.SPX_FP64, record: bool = False,
                  deriv_mode: int | None = None) -> SimulationGPU:
    """Set up one context for ``problems`` (one problem or a batch with a shared structure)."""
    if isinstance(problems, Problem):
        problems = [problems]
    base = problems[0]
    opts = dict(base.options)
    if deriv_mode is not None:
        opts[SPX_OPT_DERIV_MODE] = deriv_mode
    elif precision == capi.SPX_MIXED:
        opts[SPX_OPT_DERIV_MODE] = 1
    if record:
        opts[SPX_OPT_RECORD_FINAL] = 1
    sim = SimulationGPU(base.traj, base.time_flow, base.rk, precision, opts)
    if base.grid is not None:
        g = base.grid
        if hasattr(g, "n_blocks"):
            sim.ctx.set_background_blocks(g.n_blocks, g.domain_min, g.domain_max, g.ghost_cells, g.values)
            if g.interp_order != 1:
                sim.ctx.set_option(capi.SPX_OPT_GRID_INTERP, float(g.interp_order))
        else:
            sim.ctx.set_background_grid(g.n, g.cent_min, g.zone_length, g.values)
    for e in base.plugins:
        sim.ctx.add_plugin(e.plugin.role, e.plugin.kind, e.blob, e.n_records)
    for e in base.plugins:
        if e.plugin.role == P.ROLE_DISTRIBUTION:
            sim._distro_names.append(e.plugin.name)
            sim._distro_blobs.append(e.blob)
    for p in problems:
        sim.ctx.add_problem(p.n_traj, p.seed, _diff_overrides(base, p))
        sim._n_problems += 1
        sim._problem_distro_blobs.append({k: e.blob for k, e in enumerate(p.distributions())})
    return sim


class RunResult:
    def __init__(self, sim: SimulationGPU, stats: capi.Stats, n_problems: int, n_distros: int, records=None):
        self.stats = stats
        self.distros = [[sim.ctx.distribution(k, d) for d in range(n_distros)] for k in range(n_problems)]
        self.records = records


def run_problems(problems: list[Problem] | Problem, precision: int = capi.SPX_FP64, record: bool = False,
                 deriv_mode: int | None = None, tuning: capi.Tuning | None = None) -> RunResult:
    if isinstance(problems, Problem):
        problems = [problems]
    sim = open_problems(problems, precision, record, deriv_mode)
    try:
        stats = sim.MainLoop(tuning)
        recs = [sim.ctx.records(k, p.n_traj) for k, p in enumerate(problems)] if record else None
        return RunResult(sim, stats, len(problems), len(problems[0].distributions()), recs)
    finally:
        sim.close()
