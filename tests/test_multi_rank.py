"""The multi-GPU path of the benchmark on CPU: two gloo ranks, each with its
own flight line, combine their step times with a max reduction; the job
rate counts every rank's pairs over the slowest rank's time. No GPU."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config2(n_cells=16, n_traces=8,
                         line_offset_y=bench.line_offset(rank))
    ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
    ms_max = bench.max_over_ranks(ms, torch.device("cpu"), ws)
    pairs = sum(len(f.centers) for f in cfg.layers) * len(cfg.pos)
    out[rank] = (float(cfg.pos[0, 1]), ms_max,
                 bench.job_rate(pairs, ws, ms_max), pairs)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_fly_separate_lines_and_report_the_slowest():
    ws = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    y0, y1 = res[0][0], res[1][0]
    assert y1 - y0 == pytest.approx(200.0)
    assert res[0][1] == res[1][1] == pytest.approx(15.0)
    pairs = res[0][3]
    assert res[0][2] == pytest.approx(pairs * ws / 15e-3)
