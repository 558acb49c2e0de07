"""Per-step operation counts of the five benchmark workloads, from the op-counting build of the CPU
restatement (oracle/opcount.hh; make -C oracle opcount). Test infrastructure: it runs the oracle,
never the product.

Each workload runs a small sample in its minimal formulation (analytic field and diffusion
derivatives, deriv_mode 1); the counts of the whole run, set-up and events included, are divided
by the accepted steps. FLOP = additions + multiplications (a fused multiply-add counts 2); special
= divisions + square roots + transcendental calls, plus the Box-Muller transform's two logarithms,
two square roots, two sines and two cosines per Philox block of normals (the random streams are
counted as blocks, not as their arithmetic).

    python oracle/count_ops.py            prints the table (Markdown) and a JSON line
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_tools as ot  # noqa: E402
from spectrum_gb300 import units as U  # noqa: E402
from spectrum_gb300 import workloads as W  # noqa: E402

LIB = os.path.join(HERE, "_build", "libspx_oracle_opcount.so")


def _load():
    subprocess.run(["make", "-s", "-C", HERE, "opcount"], check=True)
    lib = ctypes.CDLL(LIB)
    lib.spx_oracle_run.restype = ctypes.c_int
    lib.spx_oracle_distro_sizes.restype = ctypes.c_int
    ot._lib = lib
    return lib


def samples():
    """(config, description, problems) of each benchmark workload, shortened to seconds of CPU."""
    return [
        (1, "pure diffusion, uniform B (Parker fwd, Euler)", [W.diffusion_uniform(n_traj=20)]),
        (2, "diffusive shock acceleration, smooth shock (Parker fwd, Euler)",
         [W.shock_acceleration(n_traj=6, x_downstream=2.0, p_max=5.0)]),
        (3, "Lorentz orbits in the dipole (RK4, 32 steps per gyro-orbit)",
         [W.dipole_orbits(n_traj=6, t_end=0.2 / U.unit_time)]),
        (4, "GCR modulation, Parker spiral (Parker bwd, Euler)",
         W.gcr_modulation(n_traj=3, energies_mev=[30.0, 300.0, 3000.0])),
        (5, "focused transport + pitch-angle scattering, Parker spiral (RK4)",
         W.focused_transport(n_problems=3, n_traj=6, t_max_hours=0.05)),
    ]


def count(problems):
    lib = ot._lib
    out = (ctypes.c_uint64 * 6)()
    lib.spx_oracle_opcount(out)  # reset
    steps = 0
    for pb in problems:
        r = ot.run_oracle(pb, deriv_mode=1)
        steps += int(r.traj["steps"].sum())
    lib.spx_oracle_opcount(out)
    add, mul, div, sqrt, trans, philox = (int(x) for x in out)
    return {"steps": steps, "flop": (add + mul) / steps, "add": add / steps, "mul": mul / steps,
            "div": div / steps, "sqrt": sqrt / steps, "trans": trans / steps, "philox_blocks": philox / steps,
            "special": (div + sqrt + trans + 8 * philox) / steps}


def main():
    _load()
    rows = []
    for cfg, desc, pbs in samples():
        c = count(pbs)
        c.update(config=cfg, workload=desc)
        rows.append(c)
    print("| Config | workload | FLOP/step | special/step | Philox blocks/step | steps counted |")
    print("|---|---|---|---|---|---|")
    for c in rows:
        print(f"| {c['config']} | {c['workload']} | {c['flop']:.1f} | {c['special']:.1f} "
              f"(div {c['div']:.1f}, sqrt {c['sqrt']:.1f}, transcendental {c['trans']:.1f}) | "
              f"{c['philox_blocks']:.3f} | {c['steps']} |")
    print(json.dumps({str(c["config"]): {k: round(v, 3) if isinstance(v, float) else v for k, v in c.items()}
                      for c in rows}))


if __name__ == "__main__":
    main()
