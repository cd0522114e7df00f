"""The replica path of bench.py --gpus N (one process per GPU, independent fits,
barrier + max of the timings over the ranks, whole-job rows/s), run here on CPU
as two gloo ranks. The estimation itself has no exchange step, so the only
collectives are the barrier and the max."""
import socket

import pytest
import torch.multiprocessing as mp

from fe_gpu_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import os

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from fe_gpu_gb300 import replicas as R

    r, w, local = R.dist_env()
    R.init(w, backend="gloo")
    R.barrier(w)
    slowest = R.max_over_ranks(1.5 + r, w)  # rank r "took" 1.5 + r seconds
    q.put((r, local, slowest, R.job_rate(1000.0, slowest, w)))
    R.barrier(w)
    R.finish(w)


def test_single_process_needs_no_group():
    assert replicas.max_over_ranks(3.25, 1) == 3.25
    replicas.barrier(1)
    assert replicas.job_rate(1000.0, 2.0, 1) == 500.0


@pytest.mark.timeout(180)
def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=150) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and [o[1] for o in out] == [0, 1]
    # every rank sees the slowest rank's time, and the job rate counts both ranks' rows
    assert all(o[2] == 2.5 for o in out)
    assert all(o[3] == pytest.approx(2 * 1000.0 / 2.5) for o in out)
