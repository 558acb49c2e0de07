"""The oracle (the C restatement in oracle/) pinned against the reference: the Philox generator
against its published known-answer vectors, the stepping path against the golden fixtures
written from the reference's own code, and -- where the reference sources were built here --
against the reference run live on inputs the fixtures do not hold. CPU only."""
import os
import sys

import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import workloads

# Random123 known-answer vectors for philox4x32-10 (counter, key, output)
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    assert ot.philox(ctr, key) == expect


def test_stream_layout():
    """Uniforms are (x + 0.5) 2^-32 of the block keyed {seed lo, seed hi} at counter
    {index, trajectory, problem, purpose << 24 | attempt}; normals are Box-Muller pairs."""
    seed, index, traj, problem, attempt = 0x0123456789ABCDEF, 7, 11, 3, 2
    key = [seed & 0xFFFFFFFF, seed >> 32]
    x_init = ot.philox([index, traj, problem, (1 << 24) | attempt], key)
    u = ot.oracle_uniforms(seed, index, traj, problem, attempt)
    assert np.array_equal(u, (np.array(x_init, dtype=np.float64) + 0.5) * 2.0 ** -32)
    x_step = np.array(ot.philox([index, traj, problem, attempt], key), dtype=np.float64)
    us = (x_step + 0.5) * 2.0 ** -32
    n = ot.oracle_normals(seed, index, traj, problem, attempt)
    r0, r1 = np.sqrt(-2 * np.log(us[0])), np.sqrt(-2 * np.log(us[2]))
    expect = [r0 * np.cos(2 * np.pi * us[1]), r0 * np.sin(2 * np.pi * us[1]),
              r1 * np.cos(2 * np.pi * us[3]), r1 * np.sin(2 * np.pi * us[3])]
    assert np.allclose(n, expect, rtol=1e-14, atol=1e-14)


# The low four status bits are the reference's object set-up state (STATE_SETUP_COMPLETE and
# friends, src/trajectory_base.cc:650), raised on every trajectory object alike; the outcome flags
# (TRAJ_FINISH .. TRAJ_DISCARD, src/trajectory_base.hh:45-57) sit above them.
OUTCOME = ~np.uint32(0xF)


def _assert_same(a: ot.OracleResult, b: ot.OracleResult):
    assert len(a.traj) == len(b.traj)
    for f in a.traj.dtype.names:
        if f == "status":
            assert np.array_equal(a.traj[f] & OUTCOME, b.traj[f] & OUTCOME), f
            continue
        assert np.array_equal(a.traj[f], b.traj[f]), f
    assert len(a.distros) == len(b.distros)
    for (ca, sa, na), (cb, sb, nb) in zip(a.distros, b.distros):
        assert na == nb
        assert np.array_equal(ca, cb)
        assert np.array_equal(sa, sb)


@pytest.mark.parametrize("name", ot.golden_names())
def test_oracle_matches_golden(name):
    """Bit-exact: every trajectory's attempts, status, steps, final and initial state and
    weights, and every distribution bin, equal the reference's output for the same spec. The
    oracle runs with its listed deviations reproduced as the reference has them (only D1, the
    smooth shock's step limit, applies to these fixtures)."""
    fx, ref = ot.load_golden(name)
    got = ot.run_oracle_golden(fx, reference_quirks=1)
    _assert_same(got, ref)


def test_oracle_smoothshock_deviation_d1():
    """Without the quirk the smooth shock's step limit uses the current shock distance (D1, the
    behaviour the CUDA kernels share): the same initial states and outcomes per trajectory, paths
    that part after the first steps near the shock."""
    fx, ref = ot.load_golden("parker_fwd_smoothshock")
    got = ot.run_oracle_golden(fx)
    for f in ("attempts", "t0", "pos0", "mom0"):
        assert np.array_equal(got.traj[f], ref.traj[f]), f
    assert np.array_equal(got.traj["status"] & OUTCOME, ref.traj["status"] & OUTCOME)
    assert np.array_equal(np.sign(got.traj["pos"][:, 0]), np.sign(ref.traj["pos"][:, 0]))
    assert not np.array_equal(got.traj["steps"], ref.traj["steps"])


def test_golden_fixtures_cover_every_trajectory_family():
    kinds = {int(ot.load_golden(n)[0]["traj_kind"]) for n in ot.golden_names()}
    assert {200, 201, 202, 203, 204, 205, 206} <= kinds


needs_ref = pytest.mark.skipif(not os.path.exists(os.path.join(ot.REF_DIR, "ref_parker_bwd_rk0")),
                               reason="reference harness not built (needs the reference sources)")


@needs_ref
def test_oracle_matches_reference_live_solarwind():
    """Fresh seed and energies the fixtures do not hold: the restatement and the reference run
    side by side."""
    pbs = workloads.gcr_modulation(n_traj=4, energies_mev=[55.0], t_max_years=0.05)
    pb = pbs[0]
    pb.seed = 0xC0FFEE
    _assert_same(ot.run_oracle(pb), ot.run_reference(pb))


needs_gc_ref = pytest.mark.skipif(not os.path.exists(os.path.join(ot.REF_DIR, "ref_guidingdiffscatt_fwd_rk25")),
                                  reason="reference harness not built (needs the reference sources)")


def _golden_builders():
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    return make_golden


@needs_gc_ref
@pytest.mark.parametrize("kind", ["guiding_dipole", "guidingscatt_slab", "guidingdiff_dipole", "guidingdiffscatt_slab",
                                  "focused_slab_reflect"])
def test_oracle_matches_reference_live_guiding(kind):
    """The guiding-centre types and focused reflection on seeds and sizes the fixtures do not hold."""
    from spectrum_gb300.problem import TRAJ_FOCUSED, TRAJ_GUIDING_DIFF, TRAJ_GUIDING_DIFF_SCATT, TRAJ_GUIDING_SCATT
    mg = _golden_builders()
    pb = {"guiding_dipole": lambda: mg._guiding_dipole(10),
          "guidingscatt_slab": lambda: mg._slab_between_mirrors(TRAJ_GUIDING_SCATT, 16, d0=2.0),
          "guidingdiff_dipole": lambda: mg._guiding_perp(TRAJ_GUIDING_DIFF, 10, dipole=True),
          "guidingdiffscatt_slab": lambda: mg._guiding_perp(TRAJ_GUIDING_DIFF_SCATT, 16, dipole=False),
          "focused_slab_reflect": lambda: mg._slab_between_mirrors(TRAJ_FOCUSED, 16, keep_records=True)}[kind]()
    pb.seed = 0xBADC0DE + len(kind)
    _assert_same(ot.run_oracle(pb), ot.run_reference(pb))


@needs_ref
def test_oracle_matches_reference_live_uniform():
    pb = workloads.diffusion_uniform(n_traj=64, kappa=0.3, t_end=0.2)
    pb.seed = 12345
    _assert_same(ot.run_oracle(pb), ot.run_reference(pb))


def test_oracle_first_offset_is_a_slice():
    """Trajectories [first, first + n) of a run are those of a run from 0 (ids key the streams)."""
    pb = workloads.diffusion_uniform(n_traj=40, t_end=0.05)
    full = ot.run_oracle(pb)
    part = ot.run_oracle(pb, first=25, n=15)
    for f in full.traj.dtype.names:
        assert np.array_equal(full.traj[f][25:], part.traj[f]), f


@needs_ref
def test_oracle_matches_reference_live_smoothshock():
    """A shock set-up the fixtures do not hold (compression 3, other seed), run by the reference and
    by the oracle with D1 reproduced: bit for bit."""
    pb = workloads.shock_acceleration(n_traj=6, s=3.0, x_escape=-1.5, x_downstream=1.5, p_max=8.0)
    pb.seed = 4242
    _assert_same(ot.run_oracle(pb, reference_quirks=1), ot.run_reference(pb))


def test_oracle_grid_of_a_uniform_field_equals_uniform_background():
    """A block holding B = (0, 0, 1) at every node gives the trajectories of BackgroundUniform:
    the interpolation weights sum to one, so only rounding separates them."""
    from spectrum_gb300.plugins import BackgroundServerCartesian
    from spectrum_gb300.problem import Grid
    pb = workloads.diffusion_uniform(n_traj=50, t_end=0.05)
    ref = ot.run_oracle(pb)
    n = 8
    grid = Grid.sample((n,) * 3, (-5.0,) * 3, (10.0 / (n - 1),) * 3,
                       lambda x, y, z: (np.zeros(x.shape + (3,)),
                                        np.stack([np.zeros_like(x), np.zeros_like(x), np.ones_like(x)], axis=-1)))
    blob_entry = pb.plugins[0]
    from spectrum_gb300.datacontainer import DataContainer
    c = DataContainer()  # the base parameters of diffusion_uniform's background (dmax0 = sqrt(2 kappa dt))
    c.double(0.0).vec((0, 0, 0)).vec((0, 0, 0)).vec((0, 0, 1.0)).double(float(np.sqrt(2.0e-3)))
    pb.plugins[0] = type(blob_entry)(BackgroundServerCartesian(), c.data(), c.size())
    pb.grid = grid
    got = ot.run_oracle(pb)
    assert np.array_equal(got.traj["steps"], ref.traj["steps"])
    assert np.allclose(got.traj["pos"], ref.traj["pos"], rtol=1e-12, atol=1e-13)
