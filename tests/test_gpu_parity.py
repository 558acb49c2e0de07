"""GPU parity: the CUDA kernels against the C restatement oracle, trajectory by trajectory, on
the same Philox streams (FP64), and distributionally for the FP32 kernels."""
import numpy as np
import pytest

import oracle_tools as ot
from spectrum_gb300 import capi, workloads
from spectrum_gb300.simulation import run_problems

pytestmark = pytest.mark.gpu

STATUS_MASK = 0x1F0


def _cmp(rec, ref, rtol):
    assert len(rec) == len(ref.traj)
    assert np.array_equal(rec["status"] & STATUS_MASK, ref.traj["status"] & STATUS_MASK)
    assert np.array_equal(rec["steps"], ref.traj["steps"])
    scale = np.maximum(np.linalg.norm(ref.traj["pos"], axis=1), 1e-30)
    err = np.max(np.linalg.norm(rec["pos"] - ref.traj["pos"], axis=1) / scale)
    assert err < rtol, err
    assert np.allclose(rec["t"], ref.traj["t"], rtol=rtol, atol=0)
    return err


def test_diffusion_uniform_fp64_matches_oracle(built_lib):
    pb = workloads.diffusion_uniform(n_traj=500)
    gpu = run_problems(pb, record=True)
    ref = ot.run_oracle(pb)
    _cmp(gpu.records[0], ref, 1e-12)
    counts, sums, nev = gpu.distros[0][0]
    rc, rs, rnev = ref.distros[0]
    assert nev == rnev == 500
    assert np.array_equal(counts, rc)
    assert np.allclose(sums[:, 0], rs[:, 0])


def test_gcr_solarwind_fp64_reference_derivatives(built_lib):
    pbs = workloads.gcr_modulation(n_traj=16, energies_mev=[100.0, 1000.0], t_max_years=0.2)
    gpu = run_problems(pbs, record=True, deriv_mode=0)
    for k, pb in enumerate(pbs):
        ref = ot.run_oracle(pb, deriv_mode=0)
        rec = gpu.records[k]
        agree = (rec["steps"] == ref.traj["steps"]) & ((rec["status"] & STATUS_MASK) == (ref.traj["status"] & STATUS_MASK))
        assert agree.mean() >= 0.9, agree
        e = np.linalg.norm(rec["pos"] - ref.traj["pos"], axis=1) / np.linalg.norm(ref.traj["pos"], axis=1)
        assert np.median(e[agree]) < 1e-6


def test_gcr_solarwind_fp64_analytic(built_lib):
    pbs = workloads.gcr_modulation(n_traj=16, energies_mev=[300.0], t_max_years=0.2)
    gpu = run_problems(pbs, record=True, deriv_mode=1)
    ref = ot.run_oracle(pbs[0], deriv_mode=1)
    rec = gpu.records[0]
    agree = (rec["steps"] == ref.traj["steps"])
    assert agree.mean() >= 0.9
    e = np.linalg.norm(rec["pos"] - ref.traj["pos"], axis=1) / np.linalg.norm(ref.traj["pos"], axis=1)
    assert np.median(e[agree]) < 1e-6


def test_diffusion_uniform_gaussian_spread(built_lib):
    # E[x^2] = E[y^2] = E[z^2] = 2 kappa t (benchmarks/benchmark_explained.txt:57-63)
    pb = workloads.diffusion_uniform(n_traj=100_000)
    for prec in (capi.SPX_FP64, capi.SPX_MIXED):
        gpu = run_problems(pb, precision=prec, record=True)
        x = gpu.records[0]["pos"]
        var = (x ** 2).mean(axis=0)
        t = gpu.records[0]["t"].mean()
        sigma = 2.0 * t * np.sqrt(2.0 / len(x))  # std of the sample second moment of N(0, 2t)
        assert np.all(np.abs(var - 2.0 * t) < 4.0 * sigma), (var, t)
