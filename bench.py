"""Benchmark of the test-particle stepping path on one GB300 (or N GPUs as independent shards).

Workload (one step = one launch over the whole batch): backward-time GCR modulation in the
Parker-spiral solar wind, 32 log-spaced energies 10 MeV - 10 GeV, lambda proportional to P^0.5
with no field dependence, kappa_perp = 0.02 kappa_par, absorbing spheres at 0.05 AU (cold) and
100 AU (LIS-weighted), and the one time boundary the reference requires 100 years back, which no
trajectory reaches (spectrum_gb300.workloads.gcr_modulation). The named job is
1e6 trajectories per energy; one step integrates ``--per-energy`` of them (by default 1e5, a tenth:
run k takes trajectory ids k*1e5 ... (k+1)*1e5 - 1 of every energy, so ten steps are the job).

Reported (one JSON line on rank 0):
  value       trajectories/s of the batched FP32 stepper (persistent work queue, float-float
              accumulation), device time of the K timed launches, descriptors already on the GPU
  fp64        the plain FP64 drop-in (one thread per trajectory) on step 0's identical Philox keys,
              its trajectories/s, and the per-bin error of the FP32 spectrum against it
  e2e         the same metric through the C ABI from host blobs to host histograms per step
  roofline    FP32 work of the dominant kernel per launch over its event-timed duration
  cpu_baseline the CPU restatement of the reference algorithm on this host's cores

``--impl reference`` times the reference algorithm on the host cores instead (the CPU
restatement in oracle/; the reference's own sources cannot be built where they are absent).
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SDE trajectories/s at <=1% bin error: batched FP32 vs plain FP64 GPU, 1 GB300"
UNIT = "trajectories/s"
WORKLOAD = "gcr_modulation_parker_spiral_32E"
# Credited work per accepted step: the reference's formulation with analytic derivatives, counted by
# the op-counting build of the CPU restatement (oracle/count_ops.py) and frozen in the benchmark spec.
FROZEN_FLOP_PER_STEP = {"gcr": 1076.0, "diffusion": 273.0, "shock": 423.0, "dipole": 1130.2, "focused": 4291.0}
FROZEN_SPECIAL_PER_STEP = {"gcr": 200.0, "diffusion": 93.0, "shock": 102.0, "dipole": 219.7, "focused": 468.0}
# Executed by the FP32 Parker solar-wind kernel (compiled for the diffusion class and the boundary
# layout of this workload) per accepted step, from the steady-state ncu capture
# (profiles/step_kernel_parker_solarwind_f32_gcr.md): FP32 operations (FFMA x 2 + FADD + FMUL) and
# thread instructions; and its DRAM bytes per trajectory (it reads no field data from HBM).
EXEC_FP32_OPS_PER_STEP = float(os.environ.get("SPX_EXEC_FP32_OPS_PER_STEP", "358"))
THREAD_INST_PER_STEP = float(os.environ.get("SPX_THREAD_INST_PER_STEP", "571"))
DRAM_BYTES_PER_TRAJ = float(os.environ.get("SPX_DRAM_BYTES_PER_TRAJ", str(55.882e6 / 320000)))
# run indices reserved per rank under torchrun: rank r integrates trajectory ids of runs
# r*RUNS_PER_RANK ... (disjoint shards of one job)
RUNS_PER_RANK = 256


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def problems(per_energy: int, seed_offset: int = 0):
    from spectrum_gb300 import workloads
    pbs = workloads.gcr_modulation(n_traj=per_energy)
    for p in pbs:
        p.seed += seed_offset
    return pbs


# ---------------------------------------------------------------------------------------------
# CPU leg (the oracle restatement of the reference algorithm) -- test infrastructure
# ---------------------------------------------------------------------------------------------
def _cpu_worker(args):
    spec_idx, first, n, per_energy = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_tools
    pbs = problems(per_energy)
    t0 = time.perf_counter()
    res = oracle_tools.run_oracle(pbs[spec_idx], first=first, n=n, deriv_mode=0, record=True)
    dt = time.perf_counter() - t0
    return int(len(res.traj)), int(res.traj["steps"].sum()), dt


class CpuLeg:
    """The reference algorithm (the C restatement with the reference's own derivative methods) on
    all host cores: one spawned process per core, tasks of two trajectories taken round-robin over
    the 32 energies (trajectories 0, 1, 2, ... of each). A sample keeps every core busy for about
    the requested wall time, then drains the tasks in flight, so the rate counts all work done in
    the measured wall time."""

    def __init__(self, per_energy: int):
        self.cores = os.cpu_count() or 1
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_tools
        oracle_tools.lib()  # build/load before starting workers
        self.pool = mp.get_context("spawn").Pool(self.cores)
        self.per_energy = per_energy
        self.k = 0
        self.n_per_task = 2

    def _task(self):
        e, rnd = self.k % 32, self.k // 32
        self.k += 1
        return (e, rnd * self.n_per_task, self.n_per_task, self.per_energy)

    def sample(self, seconds: float):
        done_traj = done_steps = 0
        t0 = time.perf_counter()
        pending = []
        while True:
            now = time.perf_counter()
            still = []
            for r in pending:
                if r.ready():
                    ntraj, nsteps, _ = r.get()
                    done_traj += ntraj
                    done_steps += nsteps
                else:
                    still.append(r)
            pending = still
            if now - t0 >= seconds:
                break
            while len(pending) < 2 * self.cores:
                pending.append(self.pool.apply_async(_cpu_worker, (self._task(),)))
            time.sleep(0.005)
        for r in pending:
            ntraj, nsteps, _ = r.get()
            done_traj += ntraj
            done_steps += nsteps
        wall = time.perf_counter() - t0
        return {"value": done_traj / wall, "unit": UNIT, "cores": self.cores, "kind": "port",
                "sample": f"{done_traj} trajectories ({done_steps} steps) of the 32-energy batch, round-robin over "
                          f"energies, {wall:.1f} s wall on {self.cores} processes",
                "steps_per_s": done_steps / wall}

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_sample(seconds: float = 20.0, per_energy: int = 1000):
    leg = CpuLeg(per_energy)
    try:
        leg.sample(min(2.0, seconds))  # workers start and load the oracle
        return leg.sample(seconds)
    finally:
        leg.close()


# ---------------------------------------------------------------------------------------------
# GPU helpers
# ---------------------------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu_index: int, path: str):
        self.path = path
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for i, n in enumerate(names):
                if r[5 + i].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(rows)}


def flush_l2(torch, dev):
    # 256 MiB > the 129 MB L2
    buf = flush_l2.buf if hasattr(flush_l2, "buf") else None
    if buf is None:
        buf = flush_l2.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    buf.zero_()
    torch.cuda.synchronize(dev)


def per_bin_error(a, b, min_count):
    """Relative per-bin differences of counts and weighted sums of two runs (a against b)."""
    worst_c = worst_s = 0.0
    nb = 0
    for (ca, sa, _), (cb, sb, _) in zip(a, b):
        m = cb >= min_count
        if not m.any():
            continue
        nb += int(m.sum())
        worst_c = max(worst_c, float((abs(ca[m].astype(float) - cb[m]) / cb[m]).max()))
        ref = sb[m, 0]
        ok = ref != 0
        if ok.any():
            worst_s = max(worst_s, float((abs(sa[m, 0][ok] - ref[ok]) / abs(ref[ok])).max()))
    return worst_c, worst_s, nb


def compare_fp32_fp64(sub, tun, tuning64, torch, dev):
    """The batched FP32 stepper against the FP64 kernel on identical Philox keys (the same problems in
    fresh contexts): both throughputs and, per energy, the relative difference of the LIS-weighted
    spectrum (the sum over the spectrum's bins) with its Monte Carlo standard error. Paths part in
    the last bits and then decorrelate, so the error of the difference is formed from the paired
    per-trajectory weights: sigma = sqrt(N var(w32 - w64)) / S64, the weights from the final records
    (an exit at the outer sphere weighs the LIS at the exit momentum, src/distribution_other.cc:567-591)."""
    import numpy as np
    from spectrum_gb300 import capi, workloads
    from spectrum_gb300.simulation import open_problems
    res = {}
    for name, prec, tn in (("fp64", capi.SPX_FP64, tuning64), ("fp32", capi.SPX_MIXED, tun)):
        s = open_problems(sub, precision=prec, deriv_mode=1, record=True)
        flush_l2(torch, dev)
        st = s.MainLoop(tn)
        recs = [s.ctx.records(k, p.n_traj) for k, p in enumerate(sub)]
        dist = [[s.ctx.distribution(k, d) for d in range(2)] for k in range(len(sub))]
        s.close()
        res[name] = (st, recs, dist)
    st64, r64, d64 = res["fp64"]
    st32, r32, d32 = res["fp32"]
    r_hot = 50.0 * workloads.ONE_AU  # between the spheres at 0.05 and 100 AU: an exit at the outer one is hot
    rows, time_bins = [], []
    for k, pb in enumerate(sub):
        s64 = float(d64[k][0][1][:, 0].sum())
        s32 = float(d32[k][0][1][:, 0].sum())
        w = []
        for rec in (r64[k], r32[k]):
            hot = np.linalg.norm(rec["pos"], axis=1) > r_hot
            w.append(np.where(hot, workloads.lis_weights(np.abs(rec["mom"][:, 0])), 0.0))
        n = len(w[0])
        e_mev = workloads.modulation_energies()[pb.problem_id]
        # the count of the spectrum's hot events (exits at the outer sphere), paired: its difference
        # between the arithmetics is the discordant pairs' difference, with sigma sqrt(n10 + n01)
        h64, h32 = w[0] > 0, w[1] > 0
        n10, n01 = int((h32 & ~h64).sum()), int((h64 & ~h32).sum())
        hot64 = int(h64.sum())
        # the exit-time histogram (outer exits, 32 bins from 0 to -t_hist, outliers into the last bin), bin by
        # bin from the records, paired: count difference and its sigma sqrt(#discordant) per bin
        t_bin = -workloads.T_HIST_YEARS * 365.0 * 24.0 * 3600.0 / workloads.U.unit_time / 32.0
        bins = [np.where(hot, np.minimum(np.floor(rec["t"] / t_bin), 31), -1).astype(int)
                for hot, rec in ((h64, r64[k]), (h32, r32[k]))]
        for b in range(32):
            c64 = int((bins[0] == b).sum())
            if c64 < 10000:
                continue
            dd = (bins[1] == b).astype(int) - (bins[0] == b).astype(int)
            time_bins.append({"energy_mev": round(e_mev, 3), "bin": b, "count_fp64": c64,
                              "count_histogram_fp64": int(d64[k][1][0][b]),
                              "rel_err": float(dd.sum()) / c64, "sigma": float(np.sqrt(np.abs(dd).sum())) / c64})
        rows.append({"energy_mev": round(e_mev, 3), "events_fp64": int(d64[k][0][2]),
                     "outer_exits_fp64": hot64,
                     "outer_exit_count_rel_err": (n10 - n01) / hot64 if hot64 else None,
                     "outer_exit_count_sigma": float(np.sqrt(n10 + n01)) / hot64 if hot64 else None,
                     "rel_err": s32 / s64 - 1.0 if s64 else None,
                     "sigma": float(np.sqrt(n * np.var(w[1] - w[0])) / s64) if s64 else None,
                     "sigma_fp64_alone": float(np.sqrt(n * np.var(w[0])) / s64) if s64 else None,
                     "records_vs_histogram": float(w[0].sum() / s64 - 1.0) if s64 else None})
    ok = [r for r in rows if r["rel_err"] is not None]
    # counts of every histogram bin with an FP64 count >= 1e4 (the criterion's bins)
    ec, _, nbins = per_bin_error([x for r in d32 for x in r], [x for r in d64 for x in r], 10000)
    return {"value": st64.trajectories / (st64.kernel_ms / 1e3), "unit": UNIT, "kernel_ms": st64.kernel_ms,
            "trajectories": st64.trajectories, "energies": [r["energy_mev"] for r in rows],
            "per_energy": sub[0].n_traj, "steps_per_s": st64.steps / (st64.kernel_ms / 1e3),
            "derivatives": "analytic (the FP32 kernel's formulation)",
            "fp32_same_batch": st32.trajectories / (st32.kernel_ms / 1e3),
            "ratio_fp32_batched_over_fp64_plain": (st32.trajectories / (st32.kernel_ms / 1e3)) /
                                                  (st64.trajectories / (st64.kernel_ms / 1e3)),
            "weighted_spectrum": rows,
            "weighted_spectrum_max_rel_err": max(abs(r["rel_err"]) for r in ok) if ok else None,
            "weighted_spectrum_max_sigma": max(r["sigma"] for r in ok) if ok else None,
            "weighted_spectrum_within_1pct": bool(ok and all(abs(r["rel_err"]) <= 0.01 for r in ok)),
            "weighted_spectrum_resolved": bool(ok and all(r["sigma"] <= 0.003 for r in ok)),
            "outer_exit_count_max_rel_err": max(abs(r["outer_exit_count_rel_err"]) for r in ok) if ok else None,
            "outer_exit_count_max_sigma": max(r["outer_exit_count_sigma"] for r in ok) if ok else None,
            "exit_time_bins": time_bins,
            "exit_time_bin_max_rel_err": max((abs(b["rel_err"]) for b in time_bins), default=None),
            "exit_time_bin_max_sigma": max((b["sigma"] for b in time_bins), default=None),
            "exit_time_bin_max_abs_z": max((abs(b["rel_err"]) / b["sigma"] for b in time_bins if b["sigma"] > 0),
                                           default=None),
            "count_bin_error": ec, "count_bins_compared": nbins}


# Throughput of the other workload families (the per-family figures). Each entry:
# builder of the problem list (FP32 run), its description, and the share of it the FP64 plain
# kernel runs for the ratio.
def _other_workloads():
    from spectrum_gb300 import units as U
    from spectrum_gb300 import workloads as W
    return {
        "diffusion": (lambda: [W.diffusion_uniform(n_traj=1_000_000)],
                      "Parker fwd, uniform B, kappa = 1, t = 1 (1,000 steps each): 1e6 trajectories "
                      "(10x the named 1e5, so one launch lasts long enough to time)", 0.1),
        "shock": (lambda: [W.shock_acceleration(n_traj=100_000, x_downstream=40.0, p_max=1.0e2)],
                  "Parker fwd, smooth shock s = 4, width 1e-3, momentum boundary 1e2 p0: 1e5 of the named 1e7 "
                  "trajectories (each makes ~3e6 steps in the shock layer; 1e5 is one trajectory per lane, so "
                  "a launch lasts as long as its longest trajectory)", 0.1),
        "dipole": (lambda: [W.dipole_orbits(n_traj=1_000_000, t_end=1.0 / U.unit_time)],
                   "Lorentz RK4 in the dipole, 1e6 protons 1-100 MeV, L 2-6, 32 steps per gyro-orbit, for 1 s "
                   "of flight (100 drift periods take ~3e8 steps for the slowest trajectory)", 0.01),
        "grid": (lambda: W.gcr_modulation_grid(n_traj=100_000, n_nodes=256),
                 "Parker bwd, the Parker spiral sampled on a 256^3 block over +-6 AU (BackgroundServerCartesian, "
                 "first-order interpolation; 537 MB of FP32 node data, above the 126 MB L2), 8 energies 30 MeV-3 GeV "
                 "x 1e5 trajectories, boundaries at 0.3 and 5 AU, 0.2 yr", 0.01),
        "guiding": (lambda: [W.guiding_dipole(n_traj=1_000_000, t_end_s=60.0)],
                    "Guiding centre RK4 in the dipole, 1e6 protons 1-100 MeV, L 2-6, pitch 10-170 deg, 60 s of "
                    "bounce and drift, mirror points recorded", 0.01),
        "focused": (lambda: W.focused_transport(n_problems=64, n_traj=20_000, t_max_hours=0.5),
                    "Focused RK4 + pitch-angle scattering, 64 problems (mean free paths 0.01-1 AU, 1-100 MeV) of "
                    "2e4 trajectories each, 0.5 h of the named 48 h", 0.05),
    }


OTHER_WORKLOADS = ("diffusion", "shock", "dipole", "focused", "grid", "guiding")
# the steady-state sample of every family: trajectories stopped after this many steps
STEADY_CAP = 4096
# families whose trajectories run millions of steps: their FP64 ratio comes from the capped sample
CAPPED_FP64 = ("shock",)


def orbit_errors(r64, r32):
    """Per trajectory of the dipole orbits, FP32 against FP64 from identical initial conditions: the
    relative |p| difference, the energy drift |p|/|p0| - 1 of each, and the error of the azimuth the
    orbit turned (radians, and relative to the turn where the turn exceeds 0.5 rad, i.e. the error of the
    drift period measured from it)."""
    import numpy as np
    same = (r64["status"] & 0x1F0) == (r32["status"] & 0x1F0)
    p64, p32 = np.linalg.norm(r64["mom"], axis=1), np.linalg.norm(r32["mom"], axis=1)
    p0 = np.linalg.norm(r64["mom0"], axis=1)
    az = lambda r: np.arctan2(r["pos"][:, 1], r["pos"][:, 0])  # noqa: E731
    az0 = np.arctan2(r64["pos0"][:, 1], r64["pos0"][:, 0])
    turn = np.mod(az0 - az(r64), 2.0 * np.pi)  # westward drift
    daz = np.abs(np.angle(np.exp(1j * (az(r32) - az(r64)))))
    fast = same & (turn > 0.5) & (turn < 6.0)
    q = lambda x: {"median": float(np.median(x)), "p99": float(np.percentile(x, 99)), "max": float(x.max())} if len(x) else None  # noqa: E731
    return {"trajectories": int(len(p64)), "same_outcome": float(same.mean()),
            "momentum_rel_diff": q(np.abs(p32 / p64 - 1.0)[same]),
            "energy_drift_fp64": q(np.abs(p64 / p0 - 1.0)), "energy_drift_fp32": q(np.abs(p32 / p0 - 1.0)),
            "azimuth_abs_diff_rad": q(daz[same]),
            "drift_period_rel_diff": q(daz[fast] / turn[fast]), "trajectories_turning_over_0.5_rad": int(fast.sum())}


def bench_other(args, rank, world, local):
    """One line per run: FP32 batched trajectories/s and steps/s of another workload family, and the
    plain FP64 kernel on a share of the same trajectories."""
    import torch
    from spectrum_gb300 import capi
    from spectrum_gb300.simulation import open_problems
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    build, desc, share = _other_workloads()[args.workload]
    pbs = build()
    sim = open_problems(pbs, precision=capi.SPX_MIXED)
    tun = sim.ctx.autotune(0)
    for _ in range(args.warmup):
        sim.MainLoop(tun)
    kms, traj, steps = [], 0, 0
    for _ in range(args.steps):
        flush_l2(torch, dev)
        st = sim.MainLoop(tun)
        kms.append(st.kernel_ms)
        traj += st.trajectories
        steps += st.steps
    steady = steady_rate(sim, tun, STEADY_CAP)
    sim.close()
    t = sum(kms) / 1e3
    line = {"metric": f"SDE trajectories/s, {args.workload} workload, batched FP32, 1 GB300",
            "value": traj / t, "unit": UNIT, "steps_per_s": steps / t, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
            "dtype": "f32 (float-float accumulation)", "data": "synthetic (seeded Philox streams)",
            "config": {"workload": args.workload, "description": desc, "problems": len(pbs),
                       "trajectories_per_step": sum(p.n_traj for p in pbs), "l2": "flushed between steps"},
            "tuning": {"block_size": tun.block_size, "steps_per_sync": tun.steps_per_sync, "schedule": tun.schedule},
            "steady_steps_per_s": steady, "steady_cap": STEADY_CAP}
    if not args.no_fp64 and args.workload in CAPPED_FP64:
        # trajectories of millions of steps: the FP64 plain kernel (one thread per trajectory) and the
        # FP32 batched kernel on the same trajectories, every one stopped after STEADY_CAP steps
        sub = build()
        for p in sub:
            p.n_traj = max(1, int(p.n_traj * share))
        rates = {}
        for name, prec, tn in (("fp64", capi.SPX_FP64, capi.Tuning(0, 0, 1, 0)), ("fp32", capi.SPX_MIXED, tun)):
            s_ = open_problems(sub, precision=prec, deriv_mode=1)
            rates[name] = steady_rate(s_, tn, STEADY_CAP, 1)
            s_.close()
        line["fp64_plain"] = {"trajectories": sum(p.n_traj for p in sub), "steps_per_s": rates["fp64"],
                              "fp32_steps_per_s_same_batch": rates["fp32"], "cap": STEADY_CAP,
                              "ratio_fp32_batched_over_fp64_plain": rates["fp32"] / rates["fp64"]}
    elif not args.no_fp64:
        sub = build()
        for p in sub:
            p.n_traj = max(1, int(p.n_traj * share))
        rec = args.workload == "dipole"
        s64 = open_problems(sub, precision=capi.SPX_FP64, deriv_mode=1, record=rec)
        flush_l2(torch, dev)
        st64 = s64.MainLoop(capi.Tuning(0, 0, 1, 0))
        r64 = [s64.ctx.records(k, p.n_traj) for k, p in enumerate(sub)] if rec else None
        s64.close()
        s32 = open_problems(sub, precision=capi.SPX_MIXED, record=rec)
        flush_l2(torch, dev)
        st32 = s32.MainLoop(tun)
        r32 = [s32.ctx.records(k, p.n_traj) for k, p in enumerate(sub)] if rec else None
        s32.close()
        line["fp64_plain"] = {"trajectories": st64.trajectories, "value": st64.trajectories / st64.kernel_ms * 1e3,
                              "steps_per_s": st64.steps / st64.kernel_ms * 1e3,
                              "ratio_fp32_batched_over_fp64_plain": (st32.trajectories / st32.kernel_ms) /
                                                                    (st64.trajectories / st64.kernel_ms)}
        if rec:
            line["fp32_vs_fp64_per_trajectory"] = orbit_errors(r64[0], r32[0])
    if rank == 0:
        print(json.dumps(line), flush=True)


def steady_rate(sim, tun, cap: int, launches: int = 3):
    """Steps/s of the batch with every trajectory stopped after ``cap`` steps: every lane busy for the
    whole launch, no drain (the best of ``launches`` launches)."""
    from spectrum_gb300 import capi
    sim.ctx.set_option(capi.SPX_OPT_STEP_CAP, cap)
    best = 0.0
    for _ in range(launches):
        st = sim.MainLoop(tun)
        best = max(best, st.steps / st.kernel_ms * 1e3)
    steady_rate.last_steps = st.steps  # accepted steps of the last launch (per-step counter figures)
    sim.ctx.set_option(capi.SPX_OPT_STEP_CAP, 0)
    return best


def bench_steady(args):
    import torch
    from spectrum_gb300 import capi
    from spectrum_gb300.simulation import open_problems
    torch.cuda.set_device(torch.device("cuda", 0))
    if args.workload == "gcr":
        pbs, name = problems(args.per_energy), WORKLOAD
    else:
        pbs, name = _other_workloads()[args.workload][0](), args.workload
    sim = open_problems(pbs, precision=capi.SPX_MIXED)
    if args.tuning:
        b, bps, sps = (int(x) for x in args.tuning.split(","))
        tun = capi.Tuning(b, bps, sps, 1)
    else:
        tun = sim.ctx.autotune(0)
    rate = steady_rate(sim, tun, args.steady, max(1, args.steps))
    sim.close()
    print(json.dumps({"metric": f"steady-state steps/s, every trajectory stopped after {args.steady} steps",
                      "workload": name, "per_energy": args.per_energy if args.workload == "gcr" else None,
                      "value": rate, "unit": "steps/s", "steps_last_launch": steady_rate.last_steps,
                      "tuning": [tun.block_size, tun.blocks_per_sm, tun.steps_per_sync]}), flush=True)


def bench_accuracy(args):
    """One JSON line: the per-bin criterion on the LIS-weighted spectrum at a sample large enough to
    resolve it (the FP64 kernel on the persistent queue: results do not depend on the schedule)."""
    import torch
    from spectrum_gb300 import capi
    from spectrum_gb300.simulation import open_problems
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    sim = open_problems(problems(args.per_energy), precision=capi.SPX_MIXED)
    tun = sim.ctx.autotune(0)
    sim.close()
    sub = problems(args.accuracy)[::8]
    t0 = time.perf_counter()
    cmp = compare_fp32_fp64(sub, tun, capi.Tuning(128, 0, 16, 1), torch, dev)
    cmp["schedule"] = "persistent work queue (both)"
    line = {"metric": "FP32 vs FP64 LIS-weighted spectrum, per-energy relative error and Monte Carlo sigma",
            "workload": WORKLOAD, "per_energy": args.accuracy, "wall_s": time.perf_counter() - t0, **cmp}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="spectrum_gb300", choices=["spectrum_gb300", "reference"])
    ap.add_argument("--per-energy", type=int, default=int(os.environ.get("SPX_BENCH_PER_ENERGY", "100000")))
    ap.add_argument("--accuracy", type=int, default=0, metavar="N",
                    help="instead of the benchmark: the FP32 stepper against the FP64 kernel (persistent queue) on "
                         "identical keys, every eighth energy x N trajectories, per-energy weighted-spectrum error "
                         "with its Monte Carlo sigma")
    ap.add_argument("--fp64-per-energy", type=int, default=4000,
                    help="trajectories per energy of the FP64 comparison (every fourth energy)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--tuning", default="", metavar="BLOCK,BLOCKS_PER_SM,STEPS_PER_SYNC",
                    help="a fixed launch shape for the persistent queue instead of the autotuner's (profiling)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--steady", type=int, default=0, metavar="CAP",
                    help="instead of the benchmark: steady-state steps/s of the batch with every trajectory stopped "
                         "after CAP steps (SPX_OPT_STEP_CAP), no drain of the queue (profiling)")
    ap.add_argument("--no-steady", action="store_true",
                    help="skip the steady-state sample (profiling: the timed launch is then the first step launch "
                         "after the warm-up)")
    ap.add_argument("--per-launch-steps", type=int, default=2,
                    help="one-slice launches timed for comparison (each pays the drain of the queue)")
    ap.add_argument("--workload", default="gcr", choices=["gcr"] + sorted(OTHER_WORKLOADS),
                    help="gcr: the headline modulation batch; the others print throughput lines for the "
                         "other workload families (shortened where the full configuration takes hours)")
    args = ap.parse_args()
    rank, world, local = rank_info()
    if args.steady:
        return bench_steady(args)
    if args.workload != "gcr":
        return bench_other(args, rank, world, local)
    if args.accuracy:
        return bench_accuracy(args)
    cfg = {"workload": WORKLOAD, "energies": 32, "per_energy": args.per_energy,
           "trajectories_per_step": 32 * args.per_energy * world, "time_flow": "backward", "background": "solar wind",
           "diffusion": "kappa_par = (0.1 AU) v/3 (R/1GV)^0.5, kappa_perp = 0.02 kappa_par",
           "kappa_b_exponent": 0.0, "kappa_perp_ratio": 0.02,
           "time_cap": "BoundaryTimeExpire 100 yr back: the reference requires one time boundary "
                       "(src/trajectory_base.cc:626-627); exits_per_energy.neither counts the trajectories that reach it",
           "boundaries": "0.05 AU absorb (cold), 100 AU absorb (LIS-weighted), 100 yr time limit",
           "fraction_of_named_job": args.per_energy / 1.0e6,
           "trajectory_ids": f"step k integrates ids k*{args.per_energy} ... (k+1)*{args.per_energy}-1 of each "
                             f"energy (rank r adds r*K*{args.per_energy}); the named job is 1e6 per energy",
           "launch": "the K timed steps run as one launch of the persistent queue over their K slices; "
                     "per_launch_per_step times one launch per slice",
           "l2": "flushed before the timed launch; the kernel reads a few KB of descriptors and keeps its state "
                 "in registers"}

    if args.impl == "reference":
        if rank != 0:
            return
        leg = CpuLeg(args.per_energy)
        try:
            for _ in range(args.warmup):  # workers start, load the oracle, reach steady state
                leg.sample(1.0)
            vals = [leg.sample(max(5.0, args.cpu_seconds / max(args.steps, 1))) for _ in range(args.steps)]
        finally:
            leg.close()
        v = sum(x["value"] for x in vals) / len(vals)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v * cfg["trajectories_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Philox streams)", "config": cfg,
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": vals[0]["cores"], "kind": "port",
                                 "sample": vals[0]["sample"]},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import numpy as np
    import torch
    from spectrum_gb300 import capi, shard
    from spectrum_gb300.simulation import open_problems

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    # ranks take disjoint trajectory-id ranges of one job (spectrum_gb300.shard)
    pbs = problems(args.per_energy)
    n_step = 32 * args.per_energy

    # ---- batched FP32 stepper: value ---------------------------------------------------------
    # Set-up (untimed) on a context of one slice: the launch shape from the project's autotuner, timed
    # on a sample of this batch, and the warm-up steps.
    sim = open_problems(pbs, precision=capi.SPX_MIXED)
    if world > 1:
        shard.assign(sim, rank, RUNS_PER_RANK)
    if args.tuning:
        b, bps, sps = (int(x) for x in args.tuning.split(","))
        tun = capi.Tuning(b, bps, sps, 1)
    else:
        tun = sim.ctx.autotune(0)
    for _ in range(args.warmup):
        sim.MainLoop(tun)
    # For comparison, not the value: one launch per slice, which pays the drain of the persistent
    # queue (the last long trajectories on nearly empty warps) once per slice.
    per_launch = None
    if args.per_launch_steps > 0:
        ms = []
        for _ in range(args.per_launch_steps):
            flush_l2(torch, dev)
            st1 = sim.MainLoop(tun)
            ms.append(st1.kernel_ms)
        per_launch = {"value": st1.trajectories * len(ms) / (sum(ms) / 1e3), "unit": UNIT, "launches": len(ms),
                      "ms_per_launch": statistics.mean(ms), "trajectories_per_launch": st1.trajectories}
    # the rate with every lane busy (trajectories stopped after 4096 steps): the bound the drain keeps
    # the whole run below
    steady = None if args.no_steady else steady_rate(sim, tun, 4096)
    sim.close()
    # The timed region: the K steps as one launch of the persistent queue over K slices. Slice k is
    # trajectory ids k*pe ... (k+1)*pe-1 of every energy (pe trajectories per energy), the ids that K
    # launches of one slice draw, so the results are the same; a job of 1e6 per energy is one launch in
    # the library too. Under torchrun rank r takes the block of K slices at run index r.
    simk = open_problems(problems(args.steps * args.per_energy), precision=capi.SPX_MIXED)
    if world > 1:
        simk.ctx.set_option(capi.SPX_OPT_RUN_INDEX, rank)
    # nvidia-smi samples of the timed region go to SPX_CLOCKS_DIR (default: the temporary directory)
    clocks_dir = os.environ.get("SPX_CLOCKS_DIR", tempfile.gettempdir())
    os.makedirs(clocks_dir, exist_ok=True)
    clocks = Clocks(local, os.path.join(clocks_dir, f"clocks_rank{rank}.csv"))
    flush_l2(torch, dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    t_wall0 = time.perf_counter()
    with clocks:
        st = simk.MainLoop(tun)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t_wall0
    steps_done, traj_done = st.steps, st.trajectories
    # where the trajectories ended: the spectrum records both spheres (the inner one cold), the
    # exit-time histogram the outer one only
    ends = [(simk.ctx.distribution(p, 1)[2], simk.ctx.distribution(p, 0)[2]) for p in range(len(pbs))]
    tuning = {"block_size": st.tuning.block_size, "blocks_per_sm": st.tuning.blocks_per_sm,
              "steps_per_sync": st.tuning.steps_per_sync,
              "schedule": "persistent work queue" if st.tuning.schedule == 1 else "one thread per trajectory",
              "chosen_by": "--tuning" if args.tuning else "spx_autotune"}
    simk.close()
    t_dev = st.kernel_ms / 1e3
    t_max = shard.max_over_ranks(t_dev) if world > 1 else t_dev
    value = traj_done * world / t_max
    steps_rate = steps_done * world / t_max

    # ---- plain FP64 drop-in on identical keys: throughput ratio and per-bin error ----------------
    fp64 = None
    if not args.no_fp64:
        # Every eighth energy, at a per-energy count that keeps the FP64 leg to about a minute; fresh
        # contexts with the same problem list draw identical Philox streams.
        sub = problems(min(args.per_energy, args.fp64_per_energy))[::8]
        fp64 = compare_fp32_fp64(sub, tun, capi.Tuning(0, 0, 1, 0), torch, dev)
        fp64["schedule"] = "one thread per trajectory"
        fp64["accuracy_note"] = ("this leg's sample times the FP64 kernel; it cannot resolve the 1% criterion "
                                 "(see the sigmas). python bench.py --accuracy 150000 compares 4 energies x 1.5e5 "
                                 "trajectories: outer-exit counts resolve it; the LIS-weighted sums, dominated by rare "
                                 "fast escapers (sigma_fp64_alone), do not at any feasible sample")

    # ---- end to end through the C ABI --------------------------------------------------------
    # A fresh context per measurement: descriptors host to device, one launch over E slices, the
    # spectra device to host. E = min(K, 4) keeps the leg short; its drain weighs more than the
    # K-slice launch's.
    n_e2e = max(1, min(args.steps, 4))
    flush_l2(torch, dev)
    t0 = time.perf_counter()
    s = open_problems(problems(n_e2e * args.per_energy), precision=capi.SPX_MIXED)
    s.ctx.set_option(capi.SPX_OPT_RUN_INDEX, world + rank)
    st_e = s.MainLoop(tun)
    outs = [s.ctx.distribution(p, 0) for p in range(len(pbs))]
    s.close()
    e2e_t = time.perf_counter() - t0
    d2h = (sum(c.nbytes + x.nbytes + 8 for c, x, _ in outs) + 64) / n_e2e
    h2d = len(pbs) * (6800 * 2) / n_e2e  # FP64 and FP32 descriptors per problem (sizeof ProblemDescT)
    e2e_val = st_e.trajectories * world / e2e_t

    # ---- roofline of the dominant kernel -------------------------------------------------------
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(dev)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, FFMA pipe
    per_gpu_steps = steps_rate / world
    ach = per_gpu_steps * FROZEN_FLOP_PER_STEP["gcr"] / 1e12
    roof = {"bound": "fp32", "unit": "TFLOP/s", "peak": fp32_peak, "achieved": ach, "frac": ach / fp32_peak,
            "peak_source": "nominal FP32 FMA pipe: SMs x 128 lanes x 2 x sm_max_mhz of MEASURED_PEAKS.json "
                           "(the file has no FP32 figure; HBM and tensor peaks do not bound this kernel)",
            "flop_per_step": FROZEN_FLOP_PER_STEP["gcr"],
            "flop_source": "credited: the reference's formulation with analytic derivatives, counted by the "
                           "op-counting CPU restatement (oracle/count_ops.py), frozen in BASELINE.md",
            "traffic": DRAM_BYTES_PER_TRAJ * traj_done,
            "traffic_unit": "bytes per launch of K slices (ncu DRAM bytes per trajectory x trajectories)"}
    # what the kernel executes: its own FP32 operations and instructions per step (ncu), which its
    # closed forms keep below the credited count
    roof["executed"] = {"fp32_ops_per_step": EXEC_FP32_OPS_PER_STEP,
                        "tflops": per_gpu_steps * EXEC_FP32_OPS_PER_STEP / 1e12,
                        "frac": per_gpu_steps * EXEC_FP32_OPS_PER_STEP / 1e12 / fp32_peak}
    # the binding resource: instruction issue (4 schedulers per SM, one warp instruction per cycle)
    issue_peak = props.multi_processor_count * 4 * sm_max * 1e6
    roof["issue"] = {"thread_inst_per_step": THREAD_INST_PER_STEP,
                     "warp_inst_per_s_at_full_simt": per_gpu_steps * THREAD_INST_PER_STEP / 32.0,
                     "peak_warp_inst_per_s": issue_peak,
                     "frac_at_full_simt": per_gpu_steps * THREAD_INST_PER_STEP / 32.0 / issue_peak}

    clk = clocks.summary()
    if ends is not None:
        n0 = args.per_energy * args.steps
        cfg["exits_per_energy"] = {"outer_100AU": [round(o / n0, 4) for o, _ in ends],
                                   "inner_0.05AU": [round((b - o) / n0, 4) for o, b in ends],
                                   "neither": [round(1.0 - b / n0, 4) for _, b in ends]}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float accumulation)",
            "data": "synthetic (seeded Philox streams)", "config": cfg, "steps_per_s": steps_rate,
            "wall_s": wall, "tuning": tuning, "gpu_launches": 1, "per_launch_per_step": per_launch,
            "steady_steps_per_s": steady,
            "fp64_plain": fp64,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roof, "clocks": clk}
    if rank == 0:
        line["cpu_baseline"] = cpu_sample(args.cpu_seconds, args.per_energy) if args.cpu_seconds > 0 else None
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
