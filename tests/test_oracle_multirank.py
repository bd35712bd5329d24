"""The reference's multi-rank program (cart_mpi.f90): decomposition, the
in-process rank group of the oracle, and the same run as two OS processes
exchanging the ghost layers over torch.distributed (gloo, world size 2)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _inp(orc, dim, nx, ny, nz):
    return orc.make_input(dim, nx, ny, nz, charlength=0.125 if dim == 2 else 0.25, xpos=0.25,
                          re=20.0, ome=1.8)


def test_decomposition_follows_setcartesian(built):
    """Hand-evaluated SetCartesian / SetLocalLength (integer arithmetic of
    cart_mpi.f90:66-80 and cart_mpi_3d.f90:68-92; ties go to the later
    candidate; the first mod(n, p) ranks get one more node)."""
    from oracle import orc
    assert orc.decompose(2, (65, 33), 1) == (1, 1)
    assert orc.decompose(2, (65, 33), 2) == (2, 1)
    assert orc.decompose(2, (65, 33), 4) == (2, 2)
    assert orc.decompose(2, (65, 33), 6) == (3, 2)
    assert orc.decompose(3, (33, 17, 17), 4) == (2, 2, 1)
    assert orc.decompose(3, (33, 17, 2), 4) == (2, 2, 1)  # no split of a 2-node z
    assert orc.local_box(2, (65, 33), (2, 2), (0, 0)) == ((33, 17), (0, 0))
    assert orc.local_box(2, (65, 33), (2, 2), (1, 1)) == ((32, 16), (33, 17))
    assert orc.local_box(3, (10, 9, 8), (3, 2, 2), (2, 1, 1)) == ((3, 4, 4), (7, 5, 4))
    with pytest.raises(ValueError):
        orc.local_box(2, (5, 33), (2, 1), (1, 0))  # 2 < ghost width: the reference aborts


def test_one_rank_group_is_the_single_rank_program(built):
    from oracle import orc
    inp = _inp(orc, 2, 64, 32, 0)
    one = orc.Oracle(inp)
    grp = orc.OracleGroup(inp, 1)
    rv = orc.r_vec(7)
    one.init_up(rv)
    one.init_pdf()
    grp.init_up(rv[None])
    grp.init_pdf()
    assert np.array_equal(one.run(0, 25, 6), grp.run(0, 25, 6))
    r = grp.ranks[0]
    for a, b in ((one.f, r.f), (one.fb, r.fb), (one.p, r.p), (one.u, r.u)):
        assert np.array_equal(a, b, equal_nan=True)


def test_ranks_tile_the_domain_and_keep_their_own_lists(built):
    from oracle import orc
    inp = _inp(orc, 2, 64, 32, 0)
    # with 17-row boxes the reference's obstacle probe (up to 17 rows above)
    # leaves some rank's array: undefined there, skipped by the oracle
    grp = orc.OracleGroup(inp, 4, allow_geom_error=True)
    assert grp.np == (2, 2)
    cover = np.zeros((33, 65), dtype=int)
    nfluid = 0
    for a, r in enumerate(grp.ranks):
        (Lx, Ly), (sx, sy) = r.local_length, r.start
        cover[sy:sy + Ly, sx:sx + Lx] += 1
        nfluid += len(r.lists["fluid_id"])
        # walls only on the ranks at the global edges
        cx, cy = grp.coords(a)
        assert (len(r.lists["bl"]) > 0) == (cx == 0)
        assert (len(r.lists["br"]) > 0) == (cx == grp.np[0] - 1)
    assert (cover == 1).all()
    assert nfluid == len(orc.Oracle(inp).lists["fluid_id"])


def test_multi_rank_run_differs_from_one_rank(built):
    """-np 2 does not reproduce -np 1 (local InitUP indices, per-rank
    obstacle scan and Monitor skip): the rank group is its own reference."""
    from oracle import orc
    inp = _inp(orc, 2, 64, 32, 0)
    rv = orc.r_vec(3)
    one = orc.Oracle(inp)
    one.init_up(rv)
    one.init_pdf()
    two = orc.OracleGroup(inp, 2)
    two.init_up(np.stack([rv, rv]))
    two.init_pdf()
    assert not np.array_equal(one.run(0, 10, 5), two.run(0, 10, 5))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, dim, n, steps, interv, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from oracle import orc, orc_dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        inp = _inp(orc, dim, *n)
        r = orc_dist.DistRank(inp, dist, allow_geom_error=True)
        r.init_up(orc.r_vec(100 + rank))
        r.init_pdf()
        log = r.run(0, steps, interv)
        np.savez(os.path.join(out, "rank%d.npz" % rank), log=log, f=r.o.f, fb=r.o.fb, p=r.o.p,
                 u=r.o.u, user=r.o.lists["b_user"])
        r.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("dim,n", [(2, (64, 32, 0)), (3, (24, 12, 12))])
def test_two_processes_over_gloo_match_the_rank_group(built, tmp_path, dim, n):
    import torch.multiprocessing as mp
    from oracle import orc
    steps, interv = 12, 5
    mp.start_processes(_worker, args=(2, _free_port(), dim, n, steps, interv, str(tmp_path)),
                       nprocs=2, join=True, start_method="spawn")
    grp = orc.OracleGroup(_inp(orc, dim, *n), 2, allow_geom_error=True)
    grp.init_up(np.stack([orc.r_vec(100), orc.r_vec(101)]))
    grp.init_pdf()
    log = grp.run(0, steps, interv)
    for a in range(2):
        d = np.load(os.path.join(tmp_path, "rank%d.npz" % a))
        r = grp.ranks[a]
        assert np.array_equal(d["log"], log)
        assert np.array_equal(d["user"], r.lists["b_user"])
        for key, ref in (("f", r.f), ("fb", r.fb), ("p", r.p), ("u", r.u)):
            assert np.array_equal(d[key], ref, equal_nan=True), key
