"""The reference's distribution dump files (DistributionTemplated::Dump, src/distribution_templated.cc:
394-425), read on the CPU. The files under tests/golden/*.out were written by the reference's own
Dump() (tests/golden/make_golden.py --dumps); these tests pin the reader and the layout the C ABI
writes against them: class name, the one Specie byte, the parameter container exactly as the
plugin blob, the event count, counts and sums exactly as the same run's histograms, and the record
arrays of a distribution that keeps records."""
import glob
import os
import struct
import sys

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import distro_file

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

DUMPS = sorted(glob.glob(os.path.join(HERE, "golden", "*.distro*.out")))
CASES = dict(make_golden.cases())


def _case_and_distro(path):
    base = os.path.basename(path)[: -len(".out")]
    name, d = base.rsplit(".distro", 1)
    return name, int(d)


def test_dump_fixtures_present():
    assert len(DUMPS) >= 5


@pytest.mark.parametrize("path", DUMPS, ids=[os.path.basename(p) for p in DUMPS])
def test_reference_dump_matches_plugin_and_histogram(path):
    name, d = _case_and_distro(path)
    pb = CASES[name]
    entry = [e for e in pb.plugins if e.plugin.role == 5][d]
    dump = distro_file.read(path)
    assert dump.class_name == entry.plugin.name
    assert dump.specie == 0
    assert dump.container == entry.blob
    assert dump.n_records == entry.n_records
    _, ref = ot.load_golden(name)
    counts, sums, n_events = ref.distros[d]
    assert dump.n_events == n_events
    assert np.array_equal(dump.counts, counts)
    assert np.array_equal(dump.sums, sums)
    if name.endswith("_records"):
        # keep_records: one record per processed event; here every event is the final state (p, mu, 0)
        assert dump.values_record.shape == (len(ref.traj), 3) and dump.weights_record.shape == (len(ref.traj), 1)
        key = lambda a: a[np.lexsort(a.T[::-1])]  # noqa: E731
        assert np.array_equal(key(dump.values_record), key(ref.traj["mom"]))
    else:
        assert dump.values_record.shape == (0, 3) and dump.weights_record.shape[0] == 0
    nb = dump.n_bins
    assert nb[0] * nb[1] * nb[2] == len(counts)


def test_some_dump_has_events():
    assert any(distro_file.read(p).n_events > 0 for p in DUMPS)


def test_truncated_dump_is_refused():
    data = open(DUMPS[0], "rb").read()
    with pytest.raises(ValueError):
        distro_file.read(data[:-3])
    with pytest.raises(ValueError):
        distro_file.read(data + b"\0")


def test_container_bins_counts_ignorable_dimensions_as_one():
    c = bytes([12]) + struct.pack("<3i", 8, 0, -1)
    assert distro_file.container_bins(c) == (8, 1, 1)
