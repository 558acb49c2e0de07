"""ctypes binding of the C ABI in include/spx.h (library: spectrum_gb300/_lib/libspx.so).

There is no fallback: if the library is missing or no sm_103 device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SPX_LIB", os.path.join(_HERE, "_lib", "libspx.so"))

SPX_OK = 0
SPX_FP64 = 0
SPX_MIXED = 1
SPX_OPT_STEPS_PER_ORBIT = 1
SPX_OPT_DERIV_MODE = 2
SPX_OPT_PA_SCATTERING = 3
SPX_OPT_RECORD_FINAL = 4
SPX_OPT_MAX_ATTEMPTS = 5
SPX_OPT_RUN_INDEX = 6
SPX_OPT_SPECIALIZE = 10
SPX_OPT_STEP_CAP = 11
SPX_OPT_GRID_INTERP = 12
SPX_OPT_RECORD_CAPACITY = 7
SPX_OPT_MU_METHOD = 8
SPX_OPT_PERP_METHOD = 9
SPX_ERR_INVALID_ARG = -1
SPX_ERR_IO = -12
SPX_ERR_MISMATCH = -14

#: the symbols include/spx.h declares
EXPORTS = ["spx_create", "spx_set_option", "spx_add_plugin", "spx_add_problem", "spx_run", "spx_sync",
           "spx_get_distribution_info", "spx_get_distribution", "spx_get_records", "spx_reset_distributions",
           "spx_dump", "spx_restore", "spx_strerror", "spx_destroy", "spx_version", "spx_run_static",
           "spx_autotune", "spx_set_background_grid", "spx_dump_distribution", "spx_restore_distribution",
           "spx_get_distribution_records", "spx_set_background_blocks", "spx_grid_units"]

#: bytes of the fixed device array spx_run_static works in (SPX_STATIC_SCRATCH_BYTES)
STATIC_SCRATCH_BYTES = 512 * 1024


class Tuning(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("steps_per_sync", ctypes.c_int),
                ("schedule", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("trajectories", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("retries", ctypes.c_int64), ("given_up", ctypes.c_int64), ("events", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int), ("tuning", Tuning)]


RECORD_DTYPE = np.dtype([("attempts", "<u4"), ("status", "<u4"), ("steps", "<u8"), ("t", "<f8"), ("pos", "<f8", 3),
                         ("mom", "<f8", 3), ("t0", "<f8"), ("pos0", "<f8", 3), ("mom0", "<f8", 3), ("amp", "<f8"),
                         ("logwgt", "<f8")])


class SpxError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} ({code})")


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing: build it with __graft_entry__.build() or "
                                    "python -m spectrum_gb300.build")
        lib = ctypes.CDLL(path)
        c_int, c_size, c_u8p, c_vp = ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p
        lib.spx_create.argtypes = [ctypes.POINTER(c_vp), c_int, c_int, c_int, c_int]
        lib.spx_set_option.argtypes = [c_vp, c_int, ctypes.c_double]
        lib.spx_add_plugin.argtypes = [c_vp, c_int, c_int, c_u8p, c_size, c_size]
        lib.spx_add_problem.argtypes = [c_vp, ctypes.c_int64, ctypes.c_uint64, c_u8p, c_size]
        lib.spx_run.argtypes = [c_vp, ctypes.POINTER(Tuning)]
        lib.spx_sync.argtypes = [c_vp, ctypes.POINTER(Stats)]
        lib.spx_get_distribution_info.argtypes = [c_vp, c_int, c_int, ctypes.POINTER(ctypes.c_int64),
                                                  ctypes.POINTER(c_int)]
        lib.spx_get_distribution.argtypes = [c_vp, c_int, c_int, c_vp, c_vp, ctypes.POINTER(ctypes.c_int64)]
        lib.spx_get_records.argtypes = [c_vp, c_int, c_vp, ctypes.c_int64]
        lib.spx_get_records.restype = ctypes.c_int64
        lib.spx_reset_distributions.argtypes = [c_vp]
        lib.spx_dump.argtypes = [c_vp, ctypes.c_char_p]
        lib.spx_restore.argtypes = [c_vp, ctypes.c_char_p]
        lib.spx_dump_distribution.argtypes = [c_vp, c_int, c_int, ctypes.c_char_p]
        lib.spx_get_distribution_records.argtypes = [c_vp, c_int, c_int, c_vp, c_vp, ctypes.c_int64,
                                                     ctypes.POINTER(ctypes.c_int64)]
        lib.spx_get_distribution_records.restype = ctypes.c_int64
        lib.spx_restore_distribution.argtypes = [c_vp, c_int, c_int, ctypes.c_char_p]
        lib.spx_strerror.argtypes = [c_int]
        lib.spx_strerror.restype = ctypes.c_char_p
        lib.spx_destroy.argtypes = [c_vp]
        lib.spx_destroy.restype = None
        lib.spx_version.restype = ctypes.c_char_p
        lib.spx_autotune.argtypes = [c_vp, ctypes.c_int64, ctypes.POINTER(Tuning)]
        lib.spx_set_background_grid.argtypes = [c_vp, c_vp, c_vp, c_vp, c_vp]
        lib.spx_set_background_blocks.argtypes = [c_vp, c_vp, c_vp, c_vp, c_int, c_vp]
        lib.spx_grid_units.argtypes = [c_vp]
        lib.spx_grid_units.restype = None
        lib.spx_run_static.argtypes = [c_vp, ctypes.POINTER(Tuning), c_vp, ctypes.c_int64, c_vp, ctypes.c_int64, c_vp,
                                       ctypes.c_int64, c_vp, ctypes.c_int64, ctypes.POINTER(Stats)]
        _lib = lib
    return _lib


def grid_units() -> np.ndarray:
    """spx_grid_units: the Fluid/Particle length, velocity and magnetic ratios and Fluid::c_code."""
    out = np.zeros(4)
    load().spx_grid_units(out.ctypes.data)
    return out


def strerror(code: int) -> str:
    try:
        return load().spx_strerror(code).decode()
    except FileNotFoundError:
        return "library not loaded"


def check(code: int, what: str) -> int:
    if code < 0:
        raise SpxError(code, what)
    return code


class Context:
    """One spx_ctx: a trajectory type, time flow, RK table and arithmetic; many problems."""

    def __init__(self, traj: int, time_flow: int, rk: int, precision: int = SPX_FP64):
        self.lib = load()
        self._h = ctypes.c_void_p()
        check(self.lib.spx_create(ctypes.byref(self._h), traj, time_flow, rk, precision), "spx_create")
        self.n_problems = 0

    def close(self) -> None:
        if self._h:
            self.lib.spx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_option(self, opt: int, value: float) -> None:
        check(self.lib.spx_set_option(self._h, opt, float(value)), "spx_set_option")

    def add_plugin(self, role: int, kind: int, blob: bytes, n_records: int = 0) -> None:
        buf = (ctypes.c_uint8 * max(len(blob), 1)).from_buffer_copy(blob or b"\0")
        check(self.lib.spx_add_plugin(self._h, role, kind, buf, len(blob), n_records), "spx_add_plugin")

    def add_problem(self, n_traj: int, seed: int, overrides: bytes = b"") -> int:
        buf = (ctypes.c_uint8 * max(len(overrides), 1)).from_buffer_copy(overrides or b"\0")
        check(self.lib.spx_add_problem(self._h, int(n_traj), int(seed) & 0xFFFFFFFFFFFFFFFF, buf, len(overrides)),
              "spx_add_problem")
        self.n_problems += 1
        return self.n_problems - 1

    def run(self, tuning: Tuning | None = None) -> None:
        check(self.lib.spx_run(self._h, ctypes.byref(tuning) if tuning is not None else None), "spx_run")

    def autotune(self, sample_traj: int = 0) -> Tuning:
        """spx_autotune: time candidate launch shapes on a sample; later runs without a tuning use
        the fastest."""
        t = Tuning()
        check(self.lib.spx_autotune(self._h, int(sample_traj), ctypes.byref(t)), "spx_autotune")
        return t

    def set_background_grid(self, n, cent_min, zone_length, values) -> None:
        """spx_set_background_grid: the block of a gridded background (values (n2, n1, n0, 6): U, B)."""
        nn = np.ascontiguousarray(np.asarray(n, dtype=np.int64))
        cm = np.ascontiguousarray(np.asarray(cent_min, dtype=np.float64))
        zl = np.ascontiguousarray(np.asarray(zone_length, dtype=np.float64))
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if v.size != 6 * int(np.prod(nn)):
            raise ValueError("values must hold 6 numbers per node")
        check(self.lib.spx_set_background_grid(self._h, nn.ctypes.data, cm.ctypes.data, zl.ctypes.data, v.ctypes.data),
              "spx_set_background_grid")

    def set_background_blocks(self, n_blocks, domain_min, domain_max, ghost_cells, values) -> None:
        """spx_set_background_blocks: the reference Cartesian reader's blocks (values: blocks x fastest, in
        each block 4^3 zones x fastest, 6 fluid-unit numbers per zone)."""
        nb = np.ascontiguousarray(np.asarray(n_blocks, dtype=np.int32))
        lo = np.ascontiguousarray(np.asarray(domain_min, dtype=np.float64))
        hi = np.ascontiguousarray(np.asarray(domain_max, dtype=np.float64))
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if v.size != 6 * 64 * int(np.prod(nb.astype(np.int64))):
            raise ValueError("values must hold 6 numbers per zone, 64 zones per block")
        check(self.lib.spx_set_background_blocks(self._h, nb.ctypes.data, lo.ctypes.data, hi.ctypes.data,
                                                 int(ghost_cells), v.ctypes.data), "spx_set_background_blocks")

    def sync(self) -> Stats:
        st = Stats()
        check(self.lib.spx_sync(self._h, ctypes.byref(st)), "spx_sync")
        return st

    def distribution_info(self, problem: int, distro: int) -> tuple[int, int]:
        nb = ctypes.c_int64()
        w = ctypes.c_int()
        check(self.lib.spx_get_distribution_info(self._h, problem, distro, ctypes.byref(nb), ctypes.byref(w)),
              "spx_get_distribution_info")
        return nb.value, w.value

    def distribution(self, problem: int, distro: int):
        nb, w = self.distribution_info(problem, distro)
        counts = np.zeros(nb, dtype=np.int32)
        sums = np.zeros(nb * w, dtype=np.float64)
        ne = ctypes.c_int64()
        check(self.lib.spx_get_distribution(self._h, problem, distro, counts.ctypes.data_as(ctypes.c_void_p),
                                            sums.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ne)),
              "spx_get_distribution")
        return counts, sums.reshape(nb, w), ne.value

    def distribution_records(self, problem: int, distro: int):
        """(values[k, 3], weights[k, width], events recorded) of a keep_records distribution
        (DistributionTemplated::AddRecord): k = min(events, SPX_OPT_RECORD_CAPACITY)."""
        _, w = self.distribution_info(problem, distro)
        total = ctypes.c_int64()
        check(self.lib.spx_get_distribution_records(self._h, problem, distro, None, None, 0, ctypes.byref(total)),
              "spx_get_distribution_records")
        n = total.value
        vals = np.zeros((max(n, 1), 3))
        wts = np.zeros((max(n, 1), w))
        k = check(self.lib.spx_get_distribution_records(self._h, problem, distro, vals.ctypes.data_as(ctypes.c_void_p),
                                                        wts.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(total)),
                  "spx_get_distribution_records")
        return vals[:k], wts[:k], total.value

    def records(self, problem: int, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=RECORD_DTYPE)
        k = check(self.lib.spx_get_records(self._h, problem, out.ctypes.data_as(ctypes.c_void_p), n),
                  "spx_get_records")
        return out[:k]

    def reset_distributions(self) -> None:
        check(self.lib.spx_reset_distributions(self._h), "spx_reset_distributions")

    def dump(self, path: str) -> None:
        check(self.lib.spx_dump(self._h, path.encode()), "spx_dump")

    def restore(self, path: str) -> None:
        check(self.lib.spx_restore(self._h, path.encode()), "spx_restore")

    def dump_distribution(self, problem: int, distro: int, path: str) -> None:
        """One distribution in the reference's dump-file layout (DistributionTemplated::Dump)."""
        check(self.lib.spx_dump_distribution(self._h, problem, distro, path.encode()), "spx_dump_distribution")

    def restore_distribution(self, problem: int, distro: int, path: str) -> None:
        """One distribution from a reference dump file (DistributionTemplated::Restore)."""
        check(self.lib.spx_restore_distribution(self._h, problem, distro, path.encode()), "spx_restore_distribution")

    def run_static(self, counts_ptr: int, n_counts: int, sums_ptr: int, n_sums: int, n_events_ptr: int,
                   n_events_len: int, records_ptr: int = 0, n_records: int = 0,
                   tuning: Tuning | None = None) -> Stats:
        """spx_run_static: one launch into caller-owned device buffers (raw device addresses), no
        device allocation by the library; blocks until done."""
        st = Stats()
        check(self.lib.spx_run_static(self._h, ctypes.byref(tuning) if tuning is not None else None,
                                      ctypes.c_void_p(counts_ptr), n_counts, ctypes.c_void_p(sums_ptr), n_sums,
                                      ctypes.c_void_p(n_events_ptr), n_events_len,
                                      ctypes.c_void_p(records_ptr) if records_ptr else None, n_records,
                                      ctypes.byref(st)), "spx_run_static")
        return st
