"""spx_run_static (the launch that allocates no device memory) against spx_run, through the C ABI:
the same context set-up, two calls in a row, per-trajectory final states and every distribution
compared. The output buffers are the caller's (allocated here by torch); the library works in its
fixed device array. Collected last so it also runs after every other GPU test in one process."""
import os
import re

import numpy as np
import pytest

from spectrum_gb300 import capi, workloads
from spectrum_gb300.simulation import open_problems

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the tolerance of the FP64 parity tests; sums differ only by atomic-add order


def _layout(ctx, problems):
    """Offsets of every (problem, distribution) in the flat output arrays, and their sizes."""
    out, oc, os_ = [], 0, 0
    for k in range(len(problems)):
        for d in range(len(problems[k].distributions())):
            nb, w = ctx.distribution_info(k, d)
            out.append((k, d, oc, os_, nb, w))
            oc += nb
            os_ += nb * w
    return out, oc, os_


@pytest.mark.parametrize("precision", [capi.SPX_MIXED, capi.SPX_FP64])
def test_run_static_matches_run(built_lib, precision):
    torch = pytest.importorskip("torch")
    pbs = workloads.gcr_modulation(n_traj=256, energies_mev=[100.0, 1000.0], t_max_years=0.1)
    ref = open_problems(pbs, precision=precision, record=True)
    sim = open_problems(pbs, precision=precision, record=True)
    try:
        layout, n_counts, n_sums = _layout(sim.ctx, pbs)
        total = sum(p.n_traj for p in pbs)
        dev = torch.device("cuda", 0)
        counts = torch.zeros(max(n_counts, 1), dtype=torch.int32, device=dev)
        sums = torch.zeros(max(n_sums, 1), dtype=torch.float64, device=dev)
        n_ev = torch.zeros(len(pbs) * 4, dtype=torch.int64, device=dev)
        recs = torch.zeros(total * capi.RECORD_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        for call in range(2):
            st_ref = ref.MainLoop()
            torch.cuda.synchronize(dev)
            free_before = torch.cuda.mem_get_info(dev)[0]
            st = sim.ctx.run_static(counts.data_ptr(), counts.numel(), sums.data_ptr(), sums.numel(), n_ev.data_ptr(),
                                    n_ev.numel(), recs.data_ptr(), total)
            torch.cuda.synchronize(dev)
            if call == 1:
                # the second call finds its array already set up on this device: nothing is allocated
                assert torch.cuda.mem_get_info(dev)[0] == free_before
            assert st.trajectories == st_ref.trajectories == total
            assert st.steps == st_ref.steps
            # per-trajectory final states of this call
            got = np.frombuffer(recs.cpu().numpy().tobytes(), dtype=capi.RECORD_DTYPE)
            first = 0
            for k, p in enumerate(pbs):
                want = ref.ctx.records(k, p.n_traj)
                mine = got[first:first + p.n_traj]
                first += p.n_traj
                for f in ("attempts", "status", "steps"):
                    assert np.array_equal(mine[f], want[f]), (call, k, f)
                for f in ("t", "pos", "mom", "t0", "pos0", "mom0", "amp", "logwgt"):
                    assert np.allclose(mine[f], want[f], rtol=RTOL, atol=0), (call, k, f)
            # distributions, accumulated over the calls so far
            c_h, s_h, e_h = counts.cpu().numpy(), sums.cpu().numpy(), n_ev.cpu().numpy()
            for k, d, oc, os_, nb, w in layout:
                rc, rs, rn = ref.ctx.distribution(k, d)
                assert np.array_equal(c_h[oc:oc + nb], rc), (call, k, d)
                assert np.allclose(s_h[os_:os_ + nb * w].reshape(nb, w), rs, rtol=RTOL, atol=0), (call, k, d)
                assert int(e_h[k * 4 + d]) == rn
    finally:
        ref.close()
        sim.close()


def _capacity():
    """The documented capacity of the fixed array, in problems per call, from include/spx.h."""
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "spx.h")).read()
    m = re.search(r"(\d+) problems in SPX_MIXED, (\d+) in SPX_FP64", hdr)
    return {capi.SPX_MIXED: int(m.group(1)), capi.SPX_FP64: int(m.group(2))}


def _static_call(torch, precision, n_problems):
    pbs = workloads.gcr_modulation(n_traj=4, energies_mev=workloads.modulation_energies(n=n_problems),
                                   t_max_years=0.01)
    sim = open_problems(pbs, precision=precision)
    try:
        dev = torch.device("cuda", 0)
        layout, n_counts, n_sums = _layout(sim.ctx, pbs)
        counts = torch.zeros(n_counts, dtype=torch.int32, device=dev)
        sums = torch.zeros(n_sums, dtype=torch.float64, device=dev)
        n_ev = torch.zeros(len(pbs) * 4, dtype=torch.int64, device=dev)
        try:
            st = sim.ctx.run_static(counts.data_ptr(), counts.numel(), sums.data_ptr(), sums.numel(),
                                    n_ev.data_ptr(), n_ev.numel())
            return st, int(counts.sum().item())
        except capi.SpxError as e:
            return e, int(counts.sum().item())
    finally:
        sim.close()


@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_run_static_accepts_its_documented_capacity(built_lib, precision):
    """Exactly as many problems as the header states fit the fixed array, and run."""
    torch = pytest.importorskip("torch")
    n = _capacity()[precision]
    st, _ = _static_call(torch, precision, n)
    assert not isinstance(st, Exception), st
    assert st.trajectories == 4 * n
    assert st.steps > 0


@pytest.mark.parametrize("precision", [capi.SPX_FP64, capi.SPX_MIXED])
def test_run_static_rejects_sizes_beyond_its_array(built_lib, precision):
    """One problem more than the header's capacity does not fit the fixed array and is refused
    before anything runs."""
    torch = pytest.importorskip("torch")
    err, events = _static_call(torch, precision, _capacity()[precision] + 1)
    assert isinstance(err, capi.SpxError)
    assert err.code == -13  # SPX_ERR_TOO_LARGE
    assert events == 0
