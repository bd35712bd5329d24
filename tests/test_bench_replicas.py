"""bench.py's replicas path (--gpus N under torchrun): the whole-job numbers
take the slowest rank's timed region and the units of all ranks. Checked
with two gloo ranks on CPU, as the driver's N>1 runs use the same code over
NCCL."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, units = bench.whole_job(10.0 + 7.5 * rank, 1000.0 * (rank + 1), True)
        np.save(os.path.join(out, "r%d.npy" % rank), np.array([ms, units]))
    finally:
        dist.destroy_process_group()


def test_whole_job_takes_slowest_rank_and_all_units(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in range(2):
        ms, units = np.load(os.path.join(tmp_path, "r%d.npy" % r))
        assert ms == 17.5 and units == 3000.0


def test_whole_job_single_rank_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job(3.0, 42, False) == (3.0, 42.0)
