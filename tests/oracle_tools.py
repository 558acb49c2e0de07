"""Test-side access to the oracles: the C restatement (oracle/_build/libspx_oracle.so) and, where
the reference sources are present, the reference itself (oracle/_ref/ref_*).

This module is test infrastructure. It is imported by tests/, by __graft_entry__.smoke() and by
the CPU-baseline leg of bench.py, and by nothing in the product package.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libspx_oracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")

TRAJ_DTYPE = np.dtype([("attempts", "<u4"), ("status", "<u4"), ("steps", "<u8"), ("t", "<f8"), ("pos", "<f8", 3),
                       ("mom", "<f8", 3), ("t0", "<f8"), ("pos0", "<f8", 3), ("mom0", "<f8", 3), ("amp", "<f8"),
                       ("logwgt", "<f8")])


class _Opts(ctypes.Structure):
    _fields_ = [("traj_type", ctypes.c_int), ("time_flow", ctypes.c_int), ("rk", ctypes.c_int),
                ("deriv_mode", ctypes.c_int), ("steps_per_orbit", ctypes.c_double),
                ("pa_scattering", ctypes.c_int), ("max_attempts", ctypes.c_int), ("reference_quirks", ctypes.c_int),
                ("mu_method", ctypes.c_int), ("perp_method", ctypes.c_int), ("nudge_libm", ctypes.c_int)]


def build_oracle() -> str:
    """Compile the C restatement (gcc only; a second or two)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)
    return ORACLE_LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        _lib = ctypes.CDLL(ORACLE_LIB)
        _lib.spx_oracle_run.restype = ctypes.c_int
        _lib.spx_oracle_distro_sizes.restype = ctypes.c_int
    return _lib


def rejections() -> int:
    """Steps an adaptive Butcher table rejected in the oracle's last run."""
    f = lib().spx_oracle_rejections
    f.restype = ctypes.c_uint64
    return int(f())


def distro_sizes(spec: bytes):
    nb = (ctypes.c_int64 * 8)()
    w = (ctypes.c_int * 8)()
    n = lib().spx_oracle_distro_sizes(spec, ctypes.c_size_t(len(spec)), 8, nb, w)
    if n < 0:
        raise ValueError("malformed spec")
    return [(int(nb[i]), int(w[i])) for i in range(n)]


class OracleResult:
    def __init__(self, traj, distros):
        self.traj = traj
        #: list of (counts int32[n], sums float64[n, width], n_events)
        self.distros = distros


def run_oracle(problem, first: int = 0, n: int | None = None, deriv_mode: int = 0, steps_per_orbit: float | None = None,
               pa_scattering: int | None = None, max_attempts: int = 100, record: bool = True,
               reference_quirks: int = 0, nudge_libm: int = 0) -> OracleResult:
    """Run the C restatement on ``problem`` (a spectrum_gb300.problem.Problem)."""
    from spectrum_gb300.workloads import (SPX_OPT_MU_METHOD, SPX_OPT_PA_SCATTERING, SPX_OPT_PERP_METHOD,
                                          SPX_OPT_STEPS_PER_ORBIT)
    if steps_per_orbit is None:
        steps_per_orbit = problem.options.get(SPX_OPT_STEPS_PER_ORBIT, 100.0)
    if pa_scattering is None:
        pa_scattering = int(problem.options.get(SPX_OPT_PA_SCATTERING, 0))
    if getattr(problem, "grid", None) is not None:
        set_grid(problem.grid)
    return run_oracle_spec(problem.to_spec(), problem.traj, problem.time_flow, problem.rk,
                           problem.n_traj if n is None else n, first=first, deriv_mode=deriv_mode,
                           steps_per_orbit=steps_per_orbit, pa_scattering=pa_scattering, max_attempts=max_attempts,
                           record=record, reference_quirks=reference_quirks,
                           mu_method=int(problem.options.get(SPX_OPT_MU_METHOD, 0)),
                           perp_method=int(problem.options.get(SPX_OPT_PERP_METHOD, 0)), nudge_libm=nudge_libm)


def run_oracle_spec(spec: bytes, traj_kind: int, time_flow: int, rk: int, n: int, first: int = 0, deriv_mode: int = 0,
                    steps_per_orbit: float = 100.0, pa_scattering: int = 0, max_attempts: int = 100,
                    record: bool = True, reference_quirks: int = 0, mu_method: int = 0,
                    perp_method: int = 0, nudge_libm: int = 0) -> OracleResult:
    """Run the C restatement on a problem spec (the bytes Problem.to_spec() makes). With
    reference_quirks=1 the listed deviations D1 and D6 are reproduced as the reference has them;
    with nudge_libm=1 every normal deviate and every transcendental function's result are one ulp
    larger in magnitude (a model of two libm implementations rounding them differently)."""
    opts = _Opts(traj_kind, time_flow, rk, deriv_mode, float(steps_per_orbit), int(pa_scattering), max_attempts,
                 int(reference_quirks), int(mu_method), int(perp_method), int(nudge_libm))
    sizes = distro_sizes(spec)
    tot = sum(s for s, _ in sizes)
    counts = np.zeros(max(tot, 1), dtype=np.int32)
    sums = np.zeros(max(sum(s * w for s, w in sizes), 1), dtype=np.float64)
    nev = np.zeros(max(len(sizes), 1), dtype=np.int64)
    traj = np.zeros(n if record else 0, dtype=TRAJ_DTYPE)
    err = ctypes.create_string_buffer(256)
    rc = lib().spx_oracle_run(spec, ctypes.c_size_t(len(spec)), ctypes.byref(opts), ctypes.c_uint32(first),
                              ctypes.c_uint32(n), traj.ctypes.data_as(ctypes.c_void_p) if record else None,
                              counts.ctypes.data_as(ctypes.c_void_p), sums.ctypes.data_as(ctypes.c_void_p),
                              nev.ctypes.data_as(ctypes.c_void_p), err, ctypes.c_size_t(256))
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}: {err.value.decode()}")
    distros = []
    off = 0
    soff = 0
    for d, (nb, w) in enumerate(sizes):
        distros.append((counts[off:off + nb].copy(), sums[soff:soff + nb * w].reshape(nb, w).copy(), int(nev[d])))
        off += nb
        soff += nb * w
    return OracleResult(traj, distros)


def grid_units() -> np.ndarray:
    """The oracle's Fluid/Particle length, velocity, magnetic ratios and Fluid::c_code."""
    out = np.zeros(4)
    lib().spx_oracle_grid_units(out.ctypes.data_as(ctypes.c_void_p))
    return out


def grid_stencil(pos):
    """The oracle's block-mode primary block and stencil of one position (None outside the domain)."""
    p = np.ascontiguousarray(np.asarray(pos, dtype=np.float64))
    node, zone = np.zeros(3, np.int32), np.zeros(3, np.int32)
    cm, zl, off, w, d = np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(8), np.zeros(24)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    if lib().spx_oracle_grid_stencil(vp(p), vp(node), vp(cm), vp(zl), vp(zone), vp(off), vp(w), vp(d)):
        return None
    return {"node": node, "cent_min": cm, "zone_length": zl, "zone": zone, "offset": off, "weights": w, "derivs": d}


def grid_fields(pos, dmax0):
    """The oracle's gridded-background fields at one point: U[3] B[3] Bmag E[3] dmax gradU[9] gradB[9]
    gradBmag[3] (None on a field error)."""
    p = np.ascontiguousarray(np.asarray(pos, dtype=np.float64))
    out = np.zeros(32)
    if lib().spx_oracle_grid_fields(p.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(dmax0),
                                    out.ctypes.data_as(ctypes.c_void_p)):
        return None
    return out


def set_grid(grid) -> None:
    """Hand a problem.Grid or problem.BlockGrid to the oracle (one grid at a time)."""
    if hasattr(grid, "n_blocks"):
        nb = np.ascontiguousarray(np.asarray(grid.n_blocks, dtype=np.int32))
        lo = np.ascontiguousarray(np.asarray(grid.domain_min, dtype=np.float64))
        hi = np.ascontiguousarray(np.asarray(grid.domain_max, dtype=np.float64))
        v = np.ascontiguousarray(np.asarray(grid.values, dtype=np.float64))
        u = grid_units()
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        lib().spx_oracle_set_grid_blocks(vp(nb), vp(lo), vp(hi), ctypes.c_int(int(grid.ghost_cells)), vp(v), vp(u))
        lib().spx_oracle_set_grid_order(ctypes.c_int(int(getattr(grid, "interp_order", 1))))
        return
    n = np.ascontiguousarray(np.asarray(grid.n, dtype=np.int64))
    cm = np.ascontiguousarray(np.asarray(grid.cent_min, dtype=np.float64))
    zl = np.ascontiguousarray(np.asarray(grid.zone_length, dtype=np.float64))
    v = np.ascontiguousarray(np.asarray(grid.values, dtype=np.float64))
    lib().spx_oracle_set_grid(n.ctypes.data_as(ctypes.c_void_p), cm.ctypes.data_as(ctypes.c_void_p),
                              zl.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p))


def philox(ctr, key):
    """Philox4x32-10 of one counter (4 words) under one key (2 words), from the oracle library."""
    out = (ctypes.c_uint32 * 4)()
    lib().spx_oracle_philox((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), out)
    return [int(x) for x in out]


# -- golden fixtures (tests/golden, written by tests/golden/make_golden.py) ----------------------
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    # trajectory fixtures (the grid fixture holds fields at points, test_oracle_grid_blocks.py; the
    # print fixture the reference's text output of distributions, test_distro_print.py)
    return sorted(f[:-4] for f in os.listdir(GOLDEN_DIR)
                  if f.endswith(".npz") and not f.startswith(("grid_", "distro_prints_")))


def load_golden(name: str):
    """(fixture dict, OracleResult of the reference's output) for one fixture."""
    fx = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    distros = []
    for d in range(int(fx["n_distros"])):
        nb, w = int(fx[f"d{d}_n_bins"]), int(fx[f"d{d}_width"])
        counts = np.zeros(nb, dtype=np.int32)
        sums = np.zeros((nb, w), dtype=np.float64)
        idx = fx[f"d{d}_idx"]
        counts[idx] = fx[f"d{d}_counts"]
        sums[idx] = fx[f"d{d}_sums"]
        distros.append((counts, sums, int(fx[f"d{d}_n_events"])))
    return fx, OracleResult(fx["traj"], distros)


def run_oracle_golden(fx, deriv_mode: int = 0, reference_quirks: int = 0) -> OracleResult:
    return run_oracle_spec(fx["spec"].tobytes(), int(fx["traj_kind"]), int(fx["time_flow"]), int(fx["rk"]),
                           int(fx["n_traj"]), deriv_mode=deriv_mode, steps_per_orbit=float(fx["steps_per_orbit"]),
                           pa_scattering=int(fx["pa_scattering"]), reference_quirks=reference_quirks,
                           mu_method=int(fx["mu_method"]) if "mu_method" in fx else 0)


def oracle_normals(seed, index, traj, problem=0, attempt=0):
    out = (ctypes.c_double * 4)()
    lib().spx_oracle_normals(ctypes.c_uint64(seed), ctypes.c_uint32(index), ctypes.c_uint32(traj),
                             ctypes.c_uint32(problem), ctypes.c_uint32(attempt), out)
    return np.array(list(out))


def oracle_uniforms(seed, index, traj, problem=0, attempt=0):
    out = (ctypes.c_double * 4)()
    lib().spx_oracle_uniforms(ctypes.c_uint64(seed), ctypes.c_uint32(index), ctypes.c_uint32(traj),
                              ctypes.c_uint32(problem), ctypes.c_uint32(attempt), out)
    return np.array(list(out))


# -- the reference itself (only where oracle/_ref was built from the reference sources) --------
REF_VARIANTS = {(206, 0, 0): "parker_fwd_rk0", (206, 1, 0): "parker_bwd_rk0", (207, 1, 0): "parkersrc_bwd_rk0",
                (200, 0, 25): "lorentz_fwd_rk25", (205, 0, 25): "focused_fwd_rk25",
                (201, 0, 25): "guiding_fwd_rk25", (202, 0, 25): "guidingscatt_fwd_rk25",
                (203, 0, 25): "guidingdiff_fwd_rk25", (204, 0, 25): "guidingdiffscatt_fwd_rk25",
                (200, 1, 25): "lorentz_bwd_rk25", (205, 1, 25): "focused_bwd_rk25", (204, 1, 25): "guidingdiffscatt_bwd_rk25",
                (207, 0, 0): "parkersrc_fwd_rk0",
                (199, 0, 25): "fieldline_fwd_rk25", (199, 1, 25): "fieldline_bwd_rk25", (199, 0, 0): "fieldline_fwd_rk0",
                (199, 0, 29): "fieldline_fwd_rk29",
                # other Butcher tables (the reference's benchmarks use 29, Dormand-Prince)
                (206, 0, 29): "parker_fwd_rk29", (206, 0, 16): "parker_fwd_rk16", (206, 1, 29): "parker_bwd_rk29",
                (207, 1, 29): "parkersrc_bwd_rk29", (205, 0, 29): "focused_fwd_rk29", (201, 0, 29): "guiding_fwd_rk29",
                (202, 0, 29): "guidingscatt_fwd_rk29", (203, 0, 29): "guidingdiff_fwd_rk29",
                **{(200, 0, rk): f"lorentz_fwd_rk{rk}" for rk in (3, 9, 12, 13, 16, 21, 26, 27, 28, 29, 31, 32)}}


def ref_binary(problem) -> str | None:
    from spectrum_gb300.workloads import SPX_OPT_MU_METHOD, SPX_OPT_PERP_METHOD
    v = REF_VARIANTS.get((problem.traj, problem.time_flow, problem.rk))
    if v is None:
        return None
    perp = int(problem.options.get(SPX_OPT_PERP_METHOD, 0))
    if perp:  # the reference compiled with that perpendicular scheme (oracle/ref_glue/perp_wrap.cc)
        if problem.traj not in (203, 204) or problem.time_flow != 0:
            return None
        v = v.replace("_fwd_", f"_perp{perp}_fwd_")
    mu = int(problem.options.get(SPX_OPT_MU_METHOD, 0))
    if mu:  # the reference compiled with that pitch-angle scheme (oracle/ref_glue/mu_wrap.cc)
        if problem.traj != 202:
            return None
        v = v.replace("guidingscatt_", f"guidingscatt_mu{mu}_")
    if any(e.plugin.name == "DistributionLossCone" for e in problem.plugins):
        v += "_bmag"  # the reference compiled with RECORD_BMAG_EXTREMA, which the loss cone reads
    path = os.path.join(REF_DIR, "ref_" + v)
    return path if os.path.exists(path) else None


def parse_ref_output(buf: bytes, sizes) -> OracleResult:
    if buf[:4] != b"SPXR":
        raise ValueError("bad reference output")
    n, nd = struct.unpack_from("<II", buf, 4)
    pos = 12
    traj = np.frombuffer(buf, dtype=TRAJ_DTYPE, count=n, offset=pos).copy()
    pos += n * TRAJ_DTYPE.itemsize
    distros = []
    for _ in range(nd):
        nb, w = struct.unpack_from("<II", buf, pos)
        pos += 8
        counts = np.frombuffer(buf, dtype=np.int32, count=nb, offset=pos).copy()
        pos += 4 * nb
        sums = np.frombuffer(buf, dtype=np.float64, count=nb * w, offset=pos).reshape(nb, w).copy()
        pos += 8 * nb * w
        (nev,) = struct.unpack_from("<i", buf, pos)
        pos += 4
        distros.append((counts, sums, nev))
    return OracleResult(traj, distros)


def run_reference(problem, timeout: float = 600.0, dump_prefix: str | None = None) -> OracleResult:
    """Run the reference's own code (oracle/_ref) on ``problem``. With ``dump_prefix``, the
    reference's DistributionTemplated::Dump also writes each distribution to <prefix><index>.out."""
    exe = ref_binary(problem)
    if exe is None:
        raise FileNotFoundError("reference harness not built for this trajectory type")
    with tempfile.TemporaryDirectory() as td:
        spec_path = os.path.join(td, "spec.bin")
        out_path = os.path.join(td, "out.bin")
        with open(spec_path, "wb") as f:
            f.write(problem.to_spec())
        cmd = [exe, spec_path, out_path] + ([dump_prefix] if dump_prefix else [])
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness failed: {r.stderr[-2000:]}")
        with open(out_path, "rb") as f:
            return parse_ref_output(f.read(), None)


# -- FP64 device parity ----------------------------------------------------------------------------
#: status bits compared between the device and the oracle (the outcome bits of the reference's TRAJ_*)
STATUS_MASK = 0x1F0
#: the FP64 kernels compute every +, -, *, / and sqrt as the oracle does (no contraction); log, exp,
#: pow, sin, cos and tanh come from CUDA's library instead of the host's, which may round the last bit
#: differently. A path's sensitivity to such differences is measured on the oracle itself: the same
#: run with every normal deviate and every transcendental result one ulp larger (nudge_libm). The
#: device must stay within this factor of that spread, or below the floor: 1e-12 relative, a few
#: thousand ulp accumulated over the 10^3-10^4 steps of these paths (the adaptive Dormand-Prince
#: guiding-centre orbits differ by 6e-13 where the nudge leaves the oracle unchanged).
CONDITIONING_FACTOR = 30.0
CONDITIONING_FLOOR = 1e-12


def rel_pos_err(a, b):
    scale = np.maximum(np.linalg.norm(b["pos"], axis=1), 1e-30)
    return np.linalg.norm(a["pos"] - b["pos"], axis=1) / scale


def assert_fp64_parity(rec, ref: OracleResult, nudged: OracleResult, distros=None):
    """Trajectory by trajectory: equal step counts and outcomes for every trajectory, and a position
    error within CONDITIONING_FACTOR times the spread a one-ulp change of the libm results makes in
    the oracle. With ``distros`` (the device's [(counts, sums, n_events), ...]) every histogram's
    counts and event count must be equal too. Returns (error, spread) per trajectory."""
    assert len(rec) == len(ref.traj)
    assert np.array_equal(rec["steps"], ref.traj["steps"]), np.flatnonzero(rec["steps"] != ref.traj["steps"])
    assert np.array_equal(rec["status"] & STATUS_MASK, ref.traj["status"] & STATUS_MASK)
    err = rel_pos_err(rec, ref.traj)
    spread = rel_pos_err(nudged.traj, ref.traj)
    bound = CONDITIONING_FACTOR * spread.max() + CONDITIONING_FLOOR
    assert err.max() <= bound, (err.max(), spread.max())
    if distros is not None:
        for d, ((c_gpu, s_gpu, n_gpu), (c_ref, s_ref, n_ref)) in enumerate(zip(distros, ref.distros)):
            assert n_gpu == n_ref, (d, n_gpu, n_ref)
            assert np.array_equal(c_gpu.astype(np.int64), c_ref.astype(np.int64))
            assert np.allclose(s_gpu, s_ref, rtol=max(bound, 1e-12), atol=1e-300, equal_nan=True)
    return err, spread
