"""Replica scaling logic of bench.py on CPU: two gloo ranks, no GPU.

The solve path does not shard inside a request (the reference's only data
exchange is the MPI halo of src/solver_mpi.f90:55-82, which is out of scope),
so N GPUs run N independent replicas: each rank takes its own seeded
workload, the timed region ends with a max-over-ranks, and the throughput is
the sum over ranks."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from specfem3d_geotech_gb300 import meshgen
    r, w, local = bench.dist()
    # each replica builds its own seeded workload (different mesh perturbations)
    mesh = meshgen.slope3d(nx=6, ny=2, nz=2, seed=1 + r)
    t_max = bench.barrier_max(0.5 + r, w)
    bench.barrier(w)
    q.put((r, w, local, float(mesh.props[:, 1].sum()), t_max))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_replicas():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=100) for _ in ps)
    for p in ps:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert [o[2] for o in out] == [0, 1]                 # local rank -> device index
    assert out[0][3] != out[1][3]                         # independent replica workloads
    assert out[0][4] == out[1][4] == 1.5                  # timed region = max over ranks
