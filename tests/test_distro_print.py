"""The reference's text output of a distribution (DistributionTemplated::Print1D, Print2D and
PrintRecords, src/distribution_templated.cc:472-686), written on the host from a distribution's
counts, sums, event count and records (spectrum_gb300.distro_print, used by
SimulationGPU.PrintDistro1D/PrintDistro2D/PrintRecords and by the C++ host mirror's methods of the
same names). Every file of tests/golden/distro_prints_ref.npz -- the reference's own Print1D of every
axis, Print2D of every pair and PrintRecords, in code and in physical units, of the distributions
whose dumps are tests/golden/*.distro<d>.out -- is reproduced byte for byte from that dump."""
import os
import subprocess

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import distro_file
from spectrum_gb300 import distro_print as dp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
PRINTS = os.path.join(GOLDEN, "distro_prints_ref.npz")


def _fixtures():
    if not os.path.exists(PRINTS):
        return {}
    f = np.load(PRINTS)
    return {k: bytes(f[k]) for k in f.files}


FIXTURES = _fixtures()
WIDTH = {"DistributionPositionCumulativeOrder1": 3, "DistributionLossCone": 3, "DistributionPositionCumulativeOrder2": 9}


def _mine(name, d, kind, dump):
    h = dp.DistroHeader.from_container(dump.container, dump.sums.shape[1])
    phys = kind.endswith("u")
    k = kind.rstrip("u")
    if k.startswith("p1d"):
        return dp.format_1d(h, dump.counts, dump.sums, dump.n_events, int(k[3]), phys)
    if k.startswith("p2d"):
        return dp.format_2d(h, dump.counts, dump.sums, dump.n_events, int(k[3]), int(k[4]), phys)
    return dp.format_records(h, dump.values_record, dump.weights_record, phys)


def test_print_fixtures_present():
    assert len(FIXTURES) >= 200


@pytest.mark.parametrize("key", sorted(FIXTURES))
def test_prints_equal_the_reference(key):
    name, rest = key.split(".distro")
    d, kind = rest.split(".")
    dump = distro_file.read(os.path.join(GOLDEN, f"{name}.distro{d}.out"))
    assert _mine(name, int(d), kind, dump).encode() == FIXTURES[key]


def test_print_edge_cases():
    """Axes out of range write nothing; equal axes of Print2D give Print1D; an empty bin prints a zero
    mean; a NaN keeps its sign as the C library prints it."""
    from spectrum_gb300.datacontainer import DataContainer as DC
    from spectrum_gb300.problem import distro_header
    c = distro_header(DC(), (2, 3, 0), (0.0, 1.0, 0.0), (1.0, 1000.0, 1.0), log_bins=(0, 1, 0)).double(1.0).double(0.0)
    h = dp.DistroHeader.from_container(c.data(), 1)
    counts = np.array([1, 0, 2, 0, 0, 3], dtype=np.int32)
    sums = np.array([[0.5], [0.0], [np.copysign(np.nan, -1.0)], [0.0], [0.0], [1.5]])
    assert dp.format_1d(h, counts, sums, 6, 3) is None and dp.format_2d(h, counts, sums, 6, 0, 3) is None
    assert dp.format_2d(h, counts, sums, 6, 1, 1) == dp.format_1d(h, counts, sums, 6, 1)
    rows = dp.format_1d(h, counts, sums, 6, 1).splitlines()
    assert rows[0] == "# Total number of events: 6" and rows[1] == ""
    # axis 1: three logarithmic bins over [1, 1000], centres 10^0.5, 10^1.5, 10^2.5; the first axis collapsed
    assert rows[2].split() == ["3.16227766", "0.5", "0.5", "1"]
    assert rows[3].split() == ["31.6227766", "0", "0", "0"]
    assert rows[4].split() == ["316.227766", "-nan", "-nan", "5"]
    assert all(len(r) == 80 for r in rows[2:])


class _FakeContext:
    """The three accessors SimulationGPU's print methods call, answering from a reference dump."""

    def __init__(self, dump):
        self.dump = dump

    def distribution_info(self, problem, distro):
        return len(self.dump.counts), self.dump.sums.shape[1]

    def distribution(self, problem, distro):
        return self.dump.counts, self.dump.sums, self.dump.n_events

    def distribution_records(self, problem, distro):
        return self.dump.values_record, self.dump.weights_record, len(self.dump.values_record)


@pytest.mark.parametrize("name", ["focused_fwd_slab_records", "guiding_fwd_dipole"])
def test_simulation_print_methods_write_the_reference_files(tmp_path, name):
    """SimulationGPU.PrintDistro1D / PrintDistro2D / PrintRecords take the binning from the
    distribution's container and the histogram from the context: fed the reference's dump, they write
    the reference's files."""
    from spectrum_gb300.simulation import SimulationGPU
    dump = distro_file.read(os.path.join(GOLDEN, f"{name}.distro0.out"))
    sim = SimulationGPU.__new__(SimulationGPU)
    sim.ctx = _FakeContext(dump)
    sim._distro_blobs = [dump.container]
    sim._problem_distro_blobs = [{}]
    for kind, call in (("p1d0", lambda p: sim.PrintDistro1D(0, 0, p)),
                       ("p1d1u", lambda p: sim.PrintDistro1D(0, 1, p, True)),
                       ("p2d01", lambda p: sim.PrintDistro2D(0, 0, 1, p)),
                       ("p2d12u", lambda p: sim.PrintDistro2D(0, 1, 2, p, True)),
                       ("prec", lambda p: sim.PrintRecords(0, p))):
        path = str(tmp_path / kind)
        call(path)
        assert open(path, "rb").read() == FIXTURES[f"{name}.distro0.{kind}"], kind


_DRIVER = r'''
#include <cstdio>
#include <string>
#include <vector>
#include "spx_simulation.hh"
// reads: u32 container bytes, container, i32 width, i64 bins, i32 counts[bins], f64 sums[bins*width],
// i64 n_events, i64 records, f64 values[3*records], f64 weights[width*records]; writes <out>.<kind>
template <class T> static void get(FILE* f, T* v, size_t n) { if (std::fread(v, sizeof(T), n, f) != n) throw 1; }
int main(int argc, char** argv)
{
   FILE* f = std::fopen(argv[1], "rb");
   uint32_t len; get(f, &len, 1);
   std::vector<uint8_t> blob(len); get(f, blob.data(), len);
   int32_t w; get(f, &w, 1);
   int64_t nb; get(f, &nb, 1);
   std::vector<int32_t> counts(nb); get(f, counts.data(), nb);
   std::vector<double> sums(nb * w); get(f, sums.data(), nb * w);
   int64_t nev, nrec; get(f, &nev, 1); get(f, &nrec, 1);
   std::vector<double> vals(3 * nrec + 1), wts(w * nrec + 1);
   get(f, vals.data(), 3 * nrec); get(f, wts.data(), w * nrec);
   std::fclose(f);
   spx::DistroLayout L;
   if (!L.Read(blob.data(), blob.size(), w)) return 3;
   const std::string out = argv[2];
   for (int u = 0; u < 2; u++) {
      const std::string us = u ? "u" : "";
      for (int k = 0; k < 3; k++) L.Print1D(out + ".p1d" + std::to_string(k) + us, counts.data(), sums.data(), nev, k, u);
      for (int a = 0; a < 3; a++)
         for (int b = a + 1; b < 3; b++)
            L.Print2D(out + ".p2d" + std::to_string(a) + std::to_string(b) + us, counts.data(), sums.data(), nev, a, b, u);
      L.PrintRecords(out + ".prec" + us, vals.data(), wts.data(), (size_t)nrec, u);
   }
   return 0;
}
'''


def test_cpp_host_mirror_prints_equal_the_reference(tmp_path):
    """spx::DistroLayout of include/spx_simulation.hh (behind SimulationGPU::PrintDistro1D, PrintDistro2D
    and PrintRecords of the C++ mirror), fed each reference dump, writes the reference's files."""
    import shutil
    import struct
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "drv.cc"
    src.write_text(_DRIVER)
    exe = str(tmp_path / "drv")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    cases = sorted({k.rsplit(".", 1)[0] for k in FIXTURES})
    for case in cases:
        dump = distro_file.read(os.path.join(GOLDEN, case + ".out"))
        w = dump.sums.shape[1]
        data = struct.pack("<I", len(dump.container)) + dump.container + struct.pack("<iq", w, len(dump.counts))
        data += dump.counts.astype("<i4").tobytes() + dump.sums.astype("<f8").tobytes()
        data += struct.pack("<qq", dump.n_events, len(dump.values_record))
        data += dump.values_record.astype("<f8").tobytes() + dump.weights_record.astype("<f8").tobytes()
        inp = tmp_path / "in.bin"
        inp.write_bytes(data)
        out = str(tmp_path / "out")
        subprocess.run([exe, str(inp), out], check=True)
        for key in [k for k in FIXTURES if k.rsplit(".", 1)[0] == case]:
            kind = key.rsplit(".", 1)[1]
            assert open(f"{out}.{kind}", "rb").read() == FIXTURES[key], key
