"""Distribution dumps through the C ABI on the device.

- spx_dump_distribution writes the reference's own file layout: for the same problem, the file
  equals the one the reference's DistributionTemplated::Dump wrote (tests/golden/*.out) in every
  field; the sums, accumulated with device atomics in another order, agree to rounding.
- spx_restore_distribution reads a reference file back: the histogram equals the file, a dump
  of it is byte-identical, and a run adds its events on top (the reference's restart,
  src/simulation.cc:714-720).
- A file of another class, a truncated or a missing file is refused with its code.
- Records (keep_records): the device appends every event's value and weight; as a set they equal the
  records in the reference's dump; dumped and restored with the histogram; beyond
  SPX_OPT_RECORD_CAPACITY events are counted and not stored.
- The whole-context checkpoint (spx_dump / spx_restore) resumes a run: restore + one run equals two
  runs in one context, since trajectory ids continue from the saved run index.
"""
import os
import sys

import numpy as np
import pytest

from spectrum_gb300 import capi, distro_file
from spectrum_gb300.simulation import open_problems, run_problems

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

CASES = dict(make_golden.cases())
DIPOLE_DUMP = os.path.join(GOLDEN, "lorentz_fwd_dipole.distro0.out")


def _dumps(name):
    return sorted(os.path.join(GOLDEN, f) for f in os.listdir(GOLDEN) if f.startswith(name + ".distro"))


def _same(a: distro_file.DistroDump, b: distro_file.DistroDump, rtol=1e-12):
    assert a.class_name == b.class_name and a.specie == b.specie
    assert a.n_records == b.n_records and a.container == b.container
    assert a.n_events == b.n_events
    assert np.array_equal(a.counts, b.counts)
    np.testing.assert_allclose(a.sums, b.sums, rtol=rtol, atol=0.0)
    assert a.values_record.shape == b.values_record.shape == (0, 3)


@pytest.mark.parametrize("name", ["lorentz_fwd_dipole", "parker_bwd_solarwind_0", "focused_fwd_solarwind"])
def test_dump_equals_reference_dump(built_lib, tmp_path, name):
    sim = open_problems(CASES[name], capi.SPX_FP64)
    try:
        sim.DistroFileName(str(tmp_path / "distro"))
        sim.MainLoop()
        for path in _dumps(name):
            d = int(os.path.basename(path).rsplit(".distro", 1)[1][:-4])
            ours = distro_file.read(sim.distro_path(d))
            _same(ours, distro_file.read(path))
    finally:
        sim.close()


def test_restore_reference_dump_then_accumulate(built_lib, tmp_path):
    pb = CASES["lorentz_fwd_dipole"]
    ref = distro_file.read(DIPOLE_DUMP)
    fresh_counts, fresh_sums, fresh_nev = run_problems(pb, capi.SPX_FP64).distros[0][0]
    sim = open_problems(pb, capi.SPX_FP64)
    try:
        sim.ctx.restore_distribution(0, 0, DIPOLE_DUMP)
        counts, sums, nev = sim.ctx.distribution(0, 0)
        assert np.array_equal(counts, ref.counts) and np.array_equal(sums, ref.sums) and nev == ref.n_events
        again = str(tmp_path / "again.out")
        sim.ctx.dump_distribution(0, 0, again)
        assert open(again, "rb").read() == open(DIPOLE_DUMP, "rb").read()
        sim.MainLoop()
        counts, sums, nev = sim.ctx.distribution(0, 0)
        assert np.array_equal(counts, ref.counts + fresh_counts)
        assert nev == ref.n_events + fresh_nev
        np.testing.assert_allclose(sums, ref.sums + fresh_sums, rtol=1e-12, atol=0.0)
    finally:
        sim.close()


def test_restore_through_the_simulation_mirror(built_lib, tmp_path):
    """RestoreDistro flags a distribution; MainLoop restores it from <prefix><d>.out and then dumps."""
    pb = CASES["lorentz_fwd_dipole"]
    prefix = str(tmp_path / "run_")
    with open(DIPOLE_DUMP, "rb") as f, open(prefix + "0.out", "wb") as g:
        g.write(f.read())
    ref = distro_file.read(DIPOLE_DUMP)
    sim = open_problems(pb, capi.SPX_FP64)
    try:
        sim.DistroFileName(prefix)
        sim.RestoreDistro(0)
        sim.MainLoop()
        out = distro_file.read(prefix + "0.out")
        assert out.n_events == 2 * ref.n_events  # the same keys again: the run repeats the reference's events
        assert np.array_equal(out.counts, 2 * ref.counts)
    finally:
        sim.close()


def _code(fn):
    with pytest.raises(capi.SpxError) as e:
        fn()
    return e.value.code


def test_restore_refuses_foreign_truncated_and_missing_files(built_lib, tmp_path):
    pb = CASES["parker_bwd_solarwind_0"]
    sim = open_problems(pb, capi.SPX_FP64)
    try:
        spectrum_dump = os.path.join(GOLDEN, "parker_bwd_solarwind_0.distro0.out")
        time_dump = os.path.join(GOLDEN, "parker_bwd_solarwind_0.distro1.out")
        # another class in the file
        assert _code(lambda: sim.ctx.restore_distribution(0, 0, time_dump)) == capi.SPX_ERR_MISMATCH
        # the same class with another parameter container (32 bins over one hour, not over 0.05 yr)
        other_times = os.path.join(GOLDEN, "focused_fwd_solarwind.distro0.out")
        assert distro_file.read(other_times).class_name == distro_file.read(time_dump).class_name
        assert _code(lambda: sim.ctx.restore_distribution(0, 1, other_times)) == capi.SPX_ERR_MISMATCH
        cut = str(tmp_path / "cut.out")
        with open(spectrum_dump, "rb") as f, open(cut, "wb") as g:
            g.write(f.read()[:-20])
        assert _code(lambda: sim.ctx.restore_distribution(0, 0, cut)) == capi.SPX_ERR_IO
        assert _code(lambda: sim.ctx.restore_distribution(0, 0, str(tmp_path / "none.out"))) == capi.SPX_ERR_IO
        assert _code(lambda: sim.ctx.restore_distribution(0, 9, spectrum_dump)) == capi.SPX_ERR_INVALID_ARG
        # the context is still usable and a good file restores
        sim.ctx.restore_distribution(0, 0, spectrum_dump)
        sim.MainLoop()
    finally:
        sim.close()


def test_checkpoint_resumes_a_run(built_lib, tmp_path):
    from spectrum_gb300 import workloads
    pb = workloads.diffusion_uniform(n_traj=2000, t_end=0.05)
    a = open_problems(pb, capi.SPX_FP64)
    b = open_problems(pb, capi.SPX_FP64)
    try:
        ckpt = str(tmp_path / "ckpt.spx")
        a.MainLoop()
        a.ctx.dump(ckpt)
        a.MainLoop()
        b.ctx.restore(ckpt)
        b.MainLoop()
        ca, sa, na = a.ctx.distribution(0, 0)
        cb, sb, nb = b.ctx.distribution(0, 0)
        assert na == nb and na >= 2000
        assert np.array_equal(ca, cb)
        np.testing.assert_allclose(sa, sb, rtol=1e-12, atol=0.0)
    finally:
        a.close()
        b.close()


def _rows(a):
    return a[np.lexsort(a.T[::-1])]


def test_records_equal_the_reference_records(built_lib, tmp_path):
    name = "focused_fwd_slab_records"
    ref = distro_file.read(os.path.join(GOLDEN, name + ".distro0.out"))
    sim = open_problems(CASES[name], capi.SPX_FP64)
    try:
        sim.DistroFileName(str(tmp_path / "rec"))
        sim.MainLoop()
        vals, wts, n = sim.ctx.distribution_records(0, 0)
        assert n == len(ref.values_record) == 12
        np.testing.assert_allclose(_rows(vals), _rows(ref.values_record), rtol=1e-12, atol=1e-14)
        np.testing.assert_array_equal(wts, ref.weights_record)
        ours = distro_file.read(sim.distro_path(0))
        np.testing.assert_allclose(_rows(ours.values_record), _rows(ref.values_record), rtol=1e-12, atol=1e-14)
        # a restored reference file brings its records back
        sim.ctx.restore_distribution(0, 0, os.path.join(GOLDEN, name + ".distro0.out"))
        vals2, wts2, n2 = sim.ctx.distribution_records(0, 0)
        assert n2 == 12
        np.testing.assert_array_equal(vals2, ref.values_record)
    finally:
        sim.close()


def test_record_capacity(built_lib, tmp_path):
    name = "focused_fwd_slab_records"
    sim = open_problems(CASES[name], capi.SPX_FP64)
    try:
        sim.ctx.set_option(capi.SPX_OPT_RECORD_CAPACITY, 5)
        sim.MainLoop()
        vals, wts, n = sim.ctx.distribution_records(0, 0)
        assert n == 12 and len(vals) == 5 and len(wts) == 5
        path = str(tmp_path / "cap.out")
        sim.ctx.dump_distribution(0, 0, path)
        assert len(distro_file.read(path).values_record) == 5
        with pytest.raises(capi.SpxError) as e:
            sim.ctx.restore_distribution(0, 0, os.path.join(GOLDEN, name + ".distro0.out"))
        assert e.value.code == -13
        # distributions without keep_records have none
        with pytest.raises(capi.SpxError) as e:
            other = open_problems(CASES["focused_fwd_slab_reflect"], capi.SPX_FP64)
            try:
                other.ctx.distribution_records(0, 0)
            finally:
                other.close()
        assert e.value.code == -8
    finally:
        sim.close()

