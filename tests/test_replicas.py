"""bench.py's multi-GPU form is replicas (each rank its own frequency, no collective on the data path): its host
logic, the per-rank frequency and the max-over-ranks step time turned into whole-job seconds per frequency, run as
two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from bench import job_seconds_per_frequency, replica_frequency
    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank, world_size=world)
    try:
        ms, value = job_seconds_per_frequency(1000.0 + 500.0 * rank, world, dist, device='cpu')
        out[rank] = (replica_frequency(1e6, rank), ms, value)
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    world = 2
    with mp.get_context('spawn').Manager() as manager:          # no fork of this multi-threaded process
        out = manager.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        results = dict(out)
    assert results[0][0] == pytest.approx(1e6) and results[1][0] == pytest.approx(1.01e6)
    for rank in range(world):
        assert results[rank][1] == pytest.approx(1500.0)             # the slowest rank's step
        assert results[rank][2] == pytest.approx(1.5 / world)         # two frequencies per step


def test_single_process_needs_no_collective():
    from bench import job_seconds_per_frequency
    assert job_seconds_per_frequency(2000.0, 1) == (2000.0, 2.0)
