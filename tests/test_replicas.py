"""Sweep points sharded over two processes (gloo on CPU): each rank runs its block of points and the
gathered result equals one run over all points. The CPU oracle stands in for each rank's GPU engine
(the sharding, the noise split and the gather are what is tested here)."""
import os

import numpy as np
import pytest

from hyburn_gb300 import replicas
from hyburn_gb300._abi import HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING, HB_SEM_NOISE_PER_POINT
from hyburn_gb300.config import MonitorConfig, Unsupported


def test_shard_bounds_cover_all_points_once():
    for n in (1, 5, 128, 129):
        for world in (1, 2, 3, 8):
            got = [replicas.shard_bounds(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [hi - lo for lo, hi in got]
            assert max(sizes) - min(sizes) <= 1


def test_batch_mean_bold_cannot_be_sharded():
    with pytest.raises(Unsupported):
        replicas.check_shardable(HB_SEM_DELAY_RING, 1, 2)
    replicas.check_shardable(HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT, 1, 2)
    replicas.check_shardable(HB_SEM_DELAY_RING, 1, 1)


def _case():
    from cases import noise_for, single_model
    mons = [MonitorConfig("Bold", tr=0.004, bold_period=10)]
    cfg = single_model("Generic2dOscillator", 16, "heun_stochastic", "Linear", (0.2,), weights="csr",
                       delays="per_edge", nsig=1e-3, monitors=mons)
    sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT | HB_SEM_NOISE_PER_POINT
    values = np.linspace(0.0, 0.3, 5).astype(np.float32)
    noise = noise_for(cfg, 90, 5, True, 3)
    return cfg, sem, values, noise


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from hyburn_gb300 import SweepParam
    from oracle.hb_oracle import OracleEngine

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg, sem, values, noise = _case()
    mine = replicas.shard_values(values, rank, world)
    eng = OracleEngine.from_config(cfg, len(mine), semantics=sem)
    local = eng.run_sweep_with_trajectory(SweepParam(-1, 0), mine, 90,
                                          noise=replicas.shard_noise(noise, len(values), sem, rank, world))
    merged = replicas.gather_result(local, 90)
    t = replicas.max_over_ranks(float(rank + 1))
    if rank == 0:
        np.savez(out_path, tavg=merged.tavg[0], fin=merged.final_states[0], traj=merged.trajectories[0],
                 bold=merged.bold[0], pv=merged.param_values, t=t, n=merged.n_sweep)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo_equal_one_engine(tmp_path):
    import socket

    import torch.multiprocessing as mp
    from hyburn_gb300 import SweepParam
    from oracle.hb_oracle import OracleEngine

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "merged.npz")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    cfg, sem, values, noise = _case()
    ref = OracleEngine.from_config(cfg, len(values), semantics=sem).run_sweep_with_trajectory(
        SweepParam(-1, 0), values, 90, noise=noise)
    assert int(got["n"]) == len(values) and float(got["t"]) == 2.0
    np.testing.assert_array_equal(got["pv"], ref.param_values)
    np.testing.assert_array_equal(got["tavg"], np.asarray(ref.tavg[0]).ravel())
    np.testing.assert_array_equal(got["fin"], np.asarray(ref.final_states[0]).ravel())
    np.testing.assert_array_equal(got["traj"], np.asarray(ref.trajectories[0]).ravel())
    np.testing.assert_array_equal(got["bold"], np.asarray(ref.bold[0]).ravel())
