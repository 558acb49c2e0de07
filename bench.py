"""Benchmark of the test-particle stepping path on one GB300 (or N GPUs as independent shards).

Workload (one step = one launch over the whole batch): backward-time GCR modulation in the
Parker-spiral solar wind, 32 log-spaced energies 10 MeV - 10 GeV, ``--per-energy`` trajectories
each, LIS-weighted spectrum at the 100 AU boundary (spectrum_gb300.workloads.gcr_modulation).

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
# Per-step work of the FP32 Parker solar-wind kernel, from one ncu capture of a 64,000-trajectory
# batch of this workload (profiles/step_kernel_parker_solarwind_f32_gcr2k.md): executed FP32
# operations (FFMA x 2 + FADD + FMUL) and thread instructions per accepted step, and DRAM bytes
# per trajectory (2.84 MB over 64,000 trajectories; the kernel reads no field data from HBM).
FP32_FLOP_PER_STEP = float(os.environ.get("SPX_FP32_FLOP_PER_STEP", "421"))
THREAD_INST_PER_STEP = 812.0
DRAM_BYTES_PER_TRAJ = 2.835e6 / 64000
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
                  "trajectories (each makes ~1e5-1e6 steps in the shock layer)", 0.01),
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
    sim.close()
    t = sum(kms) / 1e3
    line = {"metric": f"SDE trajectories/s, {args.workload} workload, batched FP32, 1 GB300",
            "value": traj / t, "unit": UNIT, "steps_per_s": steps / t, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
            "dtype": "f32 (float-float accumulation)", "data": "synthetic (seeded Philox streams)",
            "config": {"workload": args.workload, "description": desc, "problems": len(pbs),
                       "trajectories_per_step": sum(p.n_traj for p in pbs), "l2": "flushed between steps"},
            "tuning": {"block_size": tun.block_size, "steps_per_sync": tun.steps_per_sync, "schedule": tun.schedule}}
    if not args.no_fp64:
        sub = build()
        for p in sub:
            p.n_traj = max(1, int(p.n_traj * share))
        s64 = open_problems(sub, precision=capi.SPX_FP64, deriv_mode=1)
        flush_l2(torch, dev)
        st64 = s64.MainLoop(capi.Tuning(0, 0, 1, 0))
        s64.close()
        s32 = open_problems(sub, precision=capi.SPX_MIXED)
        flush_l2(torch, dev)
        st32 = s32.MainLoop(tun)
        s32.close()
        line["fp64_plain"] = {"trajectories": st64.trajectories, "value": st64.trajectories / st64.kernel_ms * 1e3,
                              "steps_per_s": st64.steps / st64.kernel_ms * 1e3,
                              "ratio_fp32_batched_over_fp64_plain": (st32.trajectories / st32.kernel_ms) /
                                                                    (st64.trajectories / st64.kernel_ms)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="spectrum_gb300", choices=["spectrum_gb300", "reference"])
    ap.add_argument("--per-energy", type=int, default=int(os.environ.get("SPX_BENCH_PER_ENERGY", "100000")))
    ap.add_argument("--fp64-per-energy", type=int, default=16000,
                    help="trajectories per energy of the FP64 comparison (every fourth energy)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", default="gcr", choices=["gcr"] + sorted(OTHER_WORKLOADS),
                    help="gcr: the headline modulation batch; the others print throughput lines for the "
                         "other workload families (shortened where the full configuration takes hours)")
    args = ap.parse_args()
    rank, world, local = rank_info()
    if args.workload != "gcr":
        return bench_other(args, rank, world, local)
    cfg = {"workload": WORKLOAD, "energies": 32, "per_energy": args.per_energy,
           "trajectories_per_step": 32 * args.per_energy * world, "time_flow": "backward", "background": "solar wind",
           "diffusion": "kappa_par = lam v/3 (R/1GV)^0.5 (B/5nT)^-1, kappa_perp = 0.02 kappa_par",
           "boundaries": "0.05 AU absorb (cold), 100 AU absorb (LIS-weighted), 1 yr", "l2": "flushed between steps"}

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
    sim = open_problems(pbs, precision=capi.SPX_MIXED)
    if world > 1:
        shard.assign(sim, rank, RUNS_PER_RANK)
    # the launch shape: the project's autotuner, timed on a sample of this batch (set-up, untimed)
    tun = sim.ctx.autotune(0)
    for _ in range(args.warmup):
        sim.MainLoop(tun)
    sim.ctx.reset_distributions()
    # nvidia-smi samples of the timed region go to SPX_CLOCKS_DIR (default: the temporary directory)
    clocks_dir = os.environ.get("SPX_CLOCKS_DIR", tempfile.gettempdir())
    os.makedirs(clocks_dir, exist_ok=True)
    clocks = Clocks(local, os.path.join(clocks_dir, f"clocks_rank{rank}.csv"))
    kms = []
    steps_done = 0
    traj_done = 0
    # the timed region: K launches, each preceded by an L2 flush, device time from CUDA events
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    t_wall0 = time.perf_counter()
    with clocks:
        first_distros = None
        for k in range(args.steps):
            flush_l2(torch, dev)
            st = sim.MainLoop(tun)
            kms.append(st.kernel_ms)
            steps_done += st.steps
            traj_done += st.trajectories
            if k == 0:
                first_distros = [sim.ctx.distribution(p, 0) for p in range(len(pbs))]
                sim.ctx.reset_distributions()
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t_wall0
    tuning = {"block_size": st.tuning.block_size, "blocks_per_sm": st.tuning.blocks_per_sm,
              "steps_per_sync": st.tuning.steps_per_sync,
              "schedule": "persistent work queue" if st.tuning.schedule == 1 else "one thread per trajectory",
              "chosen_by": "spx_autotune"}
    sim.close()
    t_dev = sum(kms) / 1e3
    t_max = shard.max_over_ranks(t_dev) if world > 1 else t_dev
    value = traj_done * world / t_max
    steps_rate = steps_done * world / t_max

    # ---- plain FP64 drop-in on step 0's keys: comparison and per-bin error -------------------
    fp64 = None
    if not args.no_fp64:
        # Every fourth energy, at a per-energy count that keeps the FP64 leg to about a minute (each
        # spectrum bin still holds >= 1e4 events); fresh contexts with the same problem list draw
        # identical Philox streams.
        sub = problems(min(args.per_energy, args.fp64_per_energy))[::4]
        sim64 = open_problems(sub, precision=capi.SPX_FP64, deriv_mode=1)
        flush_l2(torch, dev)
        st64 = sim64.MainLoop(capi.Tuning(0, 0, 1, 0))
        d64 = [[sim64.ctx.distribution(p, d) for d in range(2)] for p in range(len(sub))]
        sim64.close()
        sim32 = open_problems(sub, precision=capi.SPX_MIXED)
        flush_l2(torch, dev)
        st32 = sim32.MainLoop(tun)
        d32 = [[sim32.ctx.distribution(p, d) for d in range(2)] for p in range(len(sub))]
        sim32.close()
        # counts of every histogram (the criterion: bins with an FP64 count >= 1e4)
        ec, _, nbins = per_bin_error([x for r in d32 for x in r], [x for r in d64 for x in r], 10000)
        # the LIS-weighted spectrum (one bin per energy)
        _, es, nbs = per_bin_error([r[0] for r in d32], [r[0] for r in d64], 10000)
        fp64 = {"value": st64.trajectories / (st64.kernel_ms / 1e3), "unit": UNIT, "kernel_ms": st64.kernel_ms,
                "trajectories": st64.trajectories, "energies": "every 4th of the 32",
                "per_energy": min(args.per_energy, args.fp64_per_energy),
                "steps_per_s": st64.steps / (st64.kernel_ms / 1e3), "schedule": "one thread per trajectory",
                "derivatives": "analytic (the FP32 kernel's formulation)",
                "bin_error": ec, "bins_compared": nbins, "bin_error_ok": bool(nbins > 0 and ec <= 0.01),
                "weighted_spectrum_error": es, "weighted_bins_compared": nbs,
                "ratio_fp32_batched_over_fp64_plain": (st32.trajectories / (st32.kernel_ms / 1e3)) /
                                                      (st64.trajectories / (st64.kernel_ms / 1e3))}

    # ---- end to end through the C ABI --------------------------------------------------------
    e2e_times = []
    h2d = d2h = 0
    for k in range(max(1, min(args.steps, 2))):
        flush_l2(torch, dev)
        t0 = time.perf_counter()
        s = open_problems(pbs, precision=capi.SPX_MIXED)
        if world > 1:
            s.ctx.set_option(capi.SPX_OPT_RUN_INDEX, shard.first_run_index(rank, RUNS_PER_RANK) + RUNS_PER_RANK // 2 + k)
        st_e = s.MainLoop(tun)
        outs = [s.ctx.distribution(p, 0) for p in range(len(pbs))]
        s.close()
        e2e_times.append(time.perf_counter() - t0)
        d2h = sum(c.nbytes + x.nbytes + 8 for c, x, _ in outs) + 64
        h2d = len(pbs) * (6800 * 2)  # FP64 and FP32 descriptors per problem (sizeof ProblemDescT)
    e2e_val = st_e.trajectories * world / statistics.mean(e2e_times)

    # ---- roofline of the dominant kernel -------------------------------------------------------
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(dev)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, FFMA pipe
    roof = {"bound": "fp32", "unit": "TFLOP/s", "peak": fp32_peak,
            "peak_source": "nominal FP32 FMA pipe: SMs x 128 lanes x 2 x sm_max_mhz of MEASURED_PEAKS.json "
                           "(the file has no FP32 figure; HBM and tensor peaks do not bound this kernel)",
            "traffic": None}
    ach = steps_rate / world * FP32_FLOP_PER_STEP / 1e12
    roof.update({"achieved": ach, "frac": ach / fp32_peak, "flop_per_step": FP32_FLOP_PER_STEP,
                 "traffic": DRAM_BYTES_PER_TRAJ * traj_done / max(args.steps, 1) / world,
                 "traffic_unit": "bytes per launch (ncu, scaled by trajectories)"})
    # the binding resource: instruction issue (4 schedulers per SM, one warp instruction per cycle)
    issue_peak = props.multi_processor_count * 4 * sm_max * 1e6
    roof["issue"] = {"thread_inst_per_step": THREAD_INST_PER_STEP,
                     "warp_inst_per_s_at_full_simt": steps_rate / world * THREAD_INST_PER_STEP / 32.0,
                     "peak_warp_inst_per_s": issue_peak,
                     "frac_at_full_simt": steps_rate / world * THREAD_INST_PER_STEP / 32.0 / issue_peak}

    clk = clocks.summary()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float accumulation)",
            "data": "synthetic (seeded Philox streams)", "config": cfg, "steps_per_s": steps_rate,
            "wall_s": wall, "tuning": tuning, "gpu_launches": args.steps, "fp64_plain": fp64,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roof, "clocks": clk}
    if rank == 0:
        line["cpu_baseline"] = cpu_sample(args.cpu_seconds, args.per_energy) if args.cpu_seconds > 0 else None
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
