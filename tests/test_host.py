"""Host-side logic on the CPU: the DataContainer byte layout, problem specs, the plugin catalogue,
and the C-ABI library (it loads and exports every symbol include/spx.h declares; nothing is
launched, so no GPU is needed)."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import capi, plugins, units, workloads
from spectrum_gb300.datacontainer import DataContainer
from spectrum_gb300.problem import Problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_datacontainer_records():
    """[1-byte size][payload] per record (common/data_container.cc:139-224)."""
    c = DataContainer().double(1.5).int(-3).bool(True).vec((1.0, 2.0, 3.0)).mi((4, 5, 6))
    blob = c.data()
    assert c.size() == 5
    assert c.length() == len(blob)
    expect = (bytes([8]) + struct.pack("<d", 1.5) + bytes([4]) + struct.pack("<i", -3) + bytes([1, 1]) +
              bytes([24]) + struct.pack("<3d", 1, 2, 3) + bytes([12]) + struct.pack("<3i", 4, 5, 6))
    assert blob == expect


def test_datacontainer_record_limit():
    with pytest.raises(ValueError):
        DataContainer()._add(b"x" * 256)


def test_units_code_system():
    """Code units of common/specie.hh: c = 10 in code velocity; kinetic energy round trip."""
    p = units.mev_to_mom(100.0)
    assert abs(units.EnrKin(p) * units.unit_energy / units.MEV - 100.0) < 1e-9
    assert units.Vel(p) < 10.0


def test_problem_spec_sizes_match_oracle():
    pbs = workloads.gcr_modulation(n_traj=10, energies_mev=[100.0, 200.0, 300.0])
    sizes = ot.distro_sizes(pbs[0].to_spec())
    assert sizes == [(3 * 4, 1), (32, 1)]  # spectrum: 4 bins per energy; exit times: 32 bins
    pb = workloads.diffusion_uniform(n_traj=10)
    assert ot.distro_sizes(pb.to_spec()) == [(100 ** 3, 1)]


def test_plugin_roles_enforced():
    pb = Problem(traj=206, time_flow=0, rk=0, seed=1, n_traj=1)
    with pytest.raises(TypeError):
        pb.AddBackground(plugins.BoundaryTimeExpire(), DataContainer())


def test_workload_shapes():
    pbs = workloads.gcr_modulation(n_traj=7)
    assert len(pbs) == 32
    e = workloads.modulation_energies()
    assert abs(e[0] - 10.0) < 1e-12 and abs(e[-1] - 1.0e4) < 1e-9
    assert [p.problem_id for p in pbs] == list(range(32))
    foc = workloads.focused_transport(n_problems=64)
    counts = [p.n_traj for p in foc]
    assert min(counts) >= 1000 and max(counts) <= 1_000_000


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "spx.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char\*)\s+(spx_\w+)\s*\(", hdr, re.M)))


def test_header_and_binding_agree():
    assert _declared_symbols() == sorted(capi.EXPORTS)


def test_header_constants_match_binding():
    """Every SPX_* constant the ctypes binding (and the workload options) defines has the value of
    include/spx.h."""
    hdr = open(os.path.join(ROOT, "include", "spx.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define\s+(SPX_\w+)\s+(-?\d+)\b", hdr, re.M)}
    checked = 0
    for mod in (capi, workloads):
        for name in dir(mod):
            if name.startswith("SPX_") and isinstance(getattr(mod, name), int):
                assert name in defs, name
                assert getattr(mod, name) == defs[name], name
                checked += 1
    assert checked >= 15


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    for name in _declared_symbols():
        assert hasattr(lib, name), name
    lib.spx_strerror.restype = ctypes.c_char_p
    assert lib.spx_strerror(0) == b"success"
    lib.spx_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.spx_version()


def test_library_refuses_without_a_device(built_lib):
    """No CPU fallback: on a machine without an sm_103 device, contexts are refused."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = ctypes.CDLL(built_lib)
    lib.spx_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    h = ctypes.c_void_p()
    rc = lib.spx_create(ctypes.byref(h), 206, 0, 0, 0)
    assert rc < 0 and not h.value


def test_butcher_tables_checked_before_the_device(built_lib):
    """spx_create takes any of the reference's tables but 30 (which does not compile there); the tables
    other than Euler and RK4 in FP64 only. The checks come before the device is looked for, so a valid
    choice reaches SPX_ERR_NO_DEVICE here and an invalid one SPX_ERR_INVALID_ARG."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = ctypes.CDLL(built_lib)
    lib.spx_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    h = ctypes.c_void_p()
    fp64, mixed = 0, 1
    for traj, rk, prec, want in [(206, 29, fp64, -11), (206, 25, fp64, -11), (200, 32, fp64, -11), (205, 21, fp64, -11),
                                 (206, 0, mixed, -11), (200, 25, mixed, -11), (206, 25, mixed, -1), (200, 29, mixed, -1),
                                 (200, 30, fp64, -1), (200, 33, fp64, -1), (200, -1, fp64, -1)]:
        assert lib.spx_create(ctypes.byref(h), traj, 0, rk, prec) == want, (traj, rk, prec)


def test_record_dtype_matches_oracle():
    assert capi.RECORD_DTYPE == ot.TRAJ_DTYPE
    assert capi.RECORD_DTYPE.itemsize == 144
    assert np.dtype(capi.RECORD_DTYPE).names[0] == "attempts"


def _build_example(built_lib, tmp_path):
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "gcr_modulation")
    lib_dir = os.path.dirname(built_lib)
    # no fused multiply-add contraction (gcc's default on aarch64): the blobs' doubles must round as
    # Python's do, operation by operation
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "spectrum_gb300", "examples", "gcr_modulation.cc"), "-L", lib_dir, "-lspx",
                    f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    return exe


def test_cpp_host_mirror_blobs_equal_python(built_lib, tmp_path):
    """The C++ host mirror (include/spx_simulation.hh) writes the same parameter bytes as the
    Python builder for the modulation set-up of the example application."""
    import subprocess
    exe = _build_example(built_lib, tmp_path)
    out = subprocess.run([exe, "--dump"], check=True, capture_output=True, text=True).stdout.split("\n")
    cpp = [tuple(line.split()) for line in out if line.strip()]
    # the example follows the reference's run example: kappa ~ 1/B and a one-year time limit
    pb = workloads.gcr_modulation(n_traj=1, energies_mev=workloads.modulation_energies(4), pow_law_b=-1.0,
                                  t_max_years=1.0)[0]
    py = [(str(e.plugin.role), str(e.plugin.kind), str(e.n_records), e.blob.hex()) for e in pb.plugins]
    assert sorted(cpp) == sorted(py)
    # the same order within each role (slots are positional)
    for role in range(6):
        assert [x for x in cpp if x[0] == str(role)] == [x for x in py if x[0] == str(role)]


def test_static_capacity_matches_the_descriptor_sizes(tmp_path):
    """The capacity include/spx.h documents for spx_run_static is what its fixed array holds: the run
    counters (256 B), the FP64 descriptors and, in mixed precision, the FP32 ones at the next 256-B
    boundary (spx_capi.cu, spx_run_static), with the descriptor sizes of this build."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "sz.cc"
    src.write_text('#include <cstdio>\n#include "spx_params.hh"\n'
                   'int main() { std::printf("%zu %zu", sizeof(spx::ProblemDesc), sizeof(spx::ProblemDescT<float>)); }\n')
    exe = str(tmp_path / "sz")
    subprocess.run([gxx, "-std=c++17", "-I", os.path.join(ROOT, "spectrum_gb300", "csrc"), str(src), "-o", exe], check=True)
    pd, pr = (int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split())
    hdr = open(os.path.join(ROOT, "include", "spx.h")).read()
    scratch = 512 * 1024
    assert "#define SPX_STATIC_SCRATCH_BYTES (512u * 1024u)" in hdr
    up = lambda x: (x + 255) // 256 * 256  # noqa: E731
    fp64 = max(n for n in range(1, 1000) if 256 + pd * n <= scratch)
    mixed = max(n for n in range(1, 1000) if up(256 + pd * n) + pr * n <= scratch)
    m = re.search(r"(\d+) problems in SPX_MIXED, (\d+) in SPX_FP64", hdr)
    assert (int(m.group(1)), int(m.group(2))) == (mixed, fp64)


def test_cpp_host_mirror_has_every_plugin_class():
    """The C++ host mirror (include/spx_simulation.hh) declares one prototype per plugin class of the
    Python registry, with the same role and kind, and names every trajectory type the header defines."""
    from spectrum_gb300 import plugins as P
    from spectrum_gb300.problem import TRAJ_NAMES
    src = open(os.path.join(ROOT, "include", "spx_simulation.hh")).read()
    base_role = {"BackgroundBase": P.ROLE_BACKGROUND, "DiffusionBase": P.ROLE_DIFFUSION, "SourceBase": P.ROLE_SOURCE,
                 "BoundaryBase": P.ROLE_BOUNDARY, "InitialBase": P.ROLE_INITIAL, "DistributionBase": P.ROLE_DISTRIBUTION}
    cpp = {m.group(1): (base_role[m.group(2)], int(m.group(3)))
           for m in re.finditer(r"^SPX_PROTOTYPE\((\w+), (\w+), (\d+)\)", src, re.M)}
    py = {c.__name__: (c.role, c.kind) for c in P.all_plugins()}
    assert cpp == py
    hdr = open(os.path.join(ROOT, "include", "spx.h")).read()
    for num, name in TRAJ_NAMES.items():
        assert re.search(rf"#define SPX_TRAJ_\w+ {num}\b", hdr), num
        assert f'return "{name}";' in src, name


def test_server_data_files_read_by_both_mirrors(tmp_path):
    """AddBackground(BackgroundServerCartesian(), container, pattern) reads <pattern>.out and
    <pattern>.info as the reference's server does: the C++ mirror's CartesianData and the Python
    mirror's BlockGrid.read give the blocks the files hold, and the Python mirror hands them to
    spx_set_background_blocks."""
    import shutil
    import subprocess
    import numpy as np
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.plugins import BackgroundServerCartesian
    from spectrum_gb300.problem import BlockGrid
    from spectrum_gb300.simulation import SimulationGPU
    rng = np.random.default_rng(5)
    g = BlockGrid((2, 3, 1), (-1.5, -0.25, 0.1), (2.0, 3.0, 0.7), rng.normal(size=(6, 64, 6)), 0)
    pattern = str(tmp_path / "parker_2_3_1")
    g.write(pattern + ".out")

    calls = []

    class Ctx:
        def add_plugin(self, *a):
            pass

        def set_background_blocks(self, *a):
            calls.append(a)

    sim = SimulationGPU.__new__(SimulationGPU)
    sim.ctx = Ctx()
    sim._distro_names, sim._distro_blobs = [], []
    sim.AddBackground(BackgroundServerCartesian(), DC().double(0.0), pattern, ghost_cells=1)
    nb, lo, hi, ghost, vals = calls[0]
    assert tuple(nb) == g.n_blocks and tuple(lo) == g.domain_min and tuple(hi) == g.domain_max and ghost == 1
    assert np.array_equal(vals, g.values)

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "rd.cc"
    src.write_text('#include <cstdio>\n#include "spx_simulation.hh"\n'
                   'int main(int, char** argv) { spx::CartesianData d; if (!d.Read(argv[1])) return 3;\n'
                   '  FILE* f = std::fopen(argv[2], "wb"); std::fwrite(d.n_blocks, 4, 3, f);\n'
                   '  std::fwrite(d.domain_min, 8, 3, f); std::fwrite(d.domain_max, 8, 3, f);\n'
                   '  std::fwrite(d.values.data(), 8, d.values.size(), f); std::fclose(f); return 0; }\n')
    exe = str(tmp_path / "rd")
    subprocess.run([gxx, "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    subprocess.run([exe, pattern + ".out", str(tmp_path / "o.bin")], check=True)
    raw = open(tmp_path / "o.bin", "rb").read()
    assert np.array_equal(np.frombuffer(raw[:12], "<i4"), g.n_blocks)
    assert np.array_equal(np.frombuffer(raw[12:36], "<f8"), g.domain_min)
    assert np.array_equal(np.frombuffer(raw[36:60], "<f8"), g.domain_max)
    assert np.array_equal(np.frombuffer(raw[60:], "<f8").reshape(g.values.shape), g.values)
    assert subprocess.run([exe, str(tmp_path / "missing.out"), str(tmp_path / "x")]).returncode == 3
