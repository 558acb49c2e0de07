"""Two ranks over gloo on the CPU: each integrates its shard of trajectory ids (with the oracle
standing in for its GPU), the shards' histograms are summed with spectrum_gb300.shard, and the
sum equals one run over all trajectories. This covers the multi-rank host logic without a GPU."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, n, out_path):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    import oracle_tools as ot
    from spectrum_gb300 import shard, workloads
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pbs = [workloads.diffusion_uniform(n_traj=n, t_end=0.05),
               workloads.gcr_modulation(n_traj=n, energies_mev=[300.0], t_max_years=0.02)[0]]
        # run index r of a context = trajectory ids r*n .. r*n+n-1 of each problem
        first = shard.first_run_index(rank, 1) * n
        mine = [[d for d in ot.run_oracle(p, first=first, n=n, deriv_mode=1, record=False).distros] for p in pbs]
        total = shard.combine_distributions(mine)
        t_max = shard.max_over_ranks(float(rank + 1))
        if rank == 0:
            np.save(out_path, np.array([t_max]))
            import pickle
            with open(out_path + ".pkl", "wb") as f:
                pickle.dump(total, f)
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_sum_to_one_run(tmp_path):
    torch = pytest.importorskip("torch")
    import pickle
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_tools as ot
    from spectrum_gb300 import workloads
    ot.build_oracle()
    n = 24
    out = str(tmp_path / "rank0")
    ctx = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, n, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert float(np.load(out + ".npy")[0]) == 2.0
    with open(out + ".pkl", "rb") as f:
        total = pickle.load(f)
    pbs = [workloads.diffusion_uniform(n_traj=2 * n, t_end=0.05),
           workloads.gcr_modulation(n_traj=2 * n, energies_mev=[300.0], t_max_years=0.02)[0]]
    for k, p in enumerate(pbs):
        one = ot.run_oracle(p, n=2 * n, deriv_mode=1, record=False)
        for (c1, s1, e1), (c2, s2, e2) in zip(total[k], one.distros):
            assert e1 == e2
            assert np.array_equal(c1, c2)
            assert np.allclose(s1, s2, rtol=1e-12, atol=0)


def test_first_run_index():
    from spectrum_gb300 import shard
    assert [shard.first_run_index(r, 5) for r in range(3)] == [0, 5, 10]
    with pytest.raises(ValueError):
        shard.first_run_index(-1, 1)
