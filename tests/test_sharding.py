"""Sharded evaluation semantics with CPU ranks (gloo, world size 2): each
rank evaluates its slice of cells and stars (with the oracle, on the CPU),
the integrals and likelihood sums are composed with
milkywayathome_client_gb300.sharding over torch.distributed, and the result
must equal the full evaluation.  Also the bench's barrier / max-over-ranks
helpers under gloo."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import REPO, load_case

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _init(rank, world, port):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)


def _sharded_worker(rank, world, port, case, tmpdir, out_path):
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "tests"))
    _init(rank, world, port)
    try:
        import milkywayathome_client_gb300 as mw
        from milkywayathome_client_gb300 import sharding
        from oracle import oracle as orc
        pf, sf, g = load_case(case)
        theta = g["theta"]
        o = orc.Oracle(pf, sf)
        # integrals of this rank's slice of every area's cells (cut-subtracted)
        ints_r, _ = o.integrals(theta, rank=rank, nranks=world)
        ints = sharding.allreduce_sum(ints_r)
        composed_ints = sharding.integral_compose([ints])
        # this rank's stars, with the summed integrals
        sp = mw.StarPoints.read(sf)
        n_total = sp.number_stars
        sp.split(rank, world)
        part = os.path.join(tmpdir, f"stars_{rank}.txt")
        sp.write(part)
        orank = orc.Oracle(pf, part)
        import ctypes as C
        ps, nz, ll = C.c_double(), C.c_int(), C.c_double()
        t = np.ascontiguousarray(theta, dtype=np.float64)
        it = np.ascontiguousarray(composed_ints, dtype=np.float64)
        D = C.POINTER(C.c_double)
        orc.Oracle.lib().so_likelihood(orank._h, t.ctypes.data_as(D), it.ctypes.data_as(D), C.byref(ps),
                                       C.byref(nz), C.byref(ll), None, None)
        lk = sharding.allreduce_sum([ps.value, 0.0])
        logl = sharding.likelihood_compose([lk], n_total)
        if rank == 0:
            np.save(out_path, np.array(list(composed_ints) + [logl]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", ["three_streams", "cut_area"])
def test_sharded_composition_equals_full_evaluation(tmp_path, oracle_built, built_library, case):
    out = str(tmp_path / "out.npy")
    mp.spawn(_sharded_worker, args=(2, _free_port(), case, str(tmp_path), out), nprocs=2, join=True)
    got = np.load(out)
    pf, sf, g = load_case(case)
    full = oracle_built.Oracle(pf, sf).evaluate(g["theta"])
    want = [full["background_integral"]] + list(full["stream_integrals"])
    np.testing.assert_allclose(got[:-1], want, rtol=1e-12)
    assert abs(got[-1] - full["likelihood"]) <= 1e-12


def _bench_helpers_worker(rank, world, port, out_path):
    sys.path.insert(0, REPO)
    _init(rank, world, port)
    try:
        import bench
        bench.barrier(world)
        m = bench.allreduce_max(world, 10.0 + rank)
        if rank == 0:
            np.save(out_path, np.array([m]))
    finally:
        dist.destroy_process_group()


def test_bench_max_over_ranks(tmp_path):
    out = str(tmp_path / "m.npy")
    mp.spawn(_bench_helpers_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    assert float(np.load(out)[0]) == 11.0


def test_slice_bounds_partition():
    from milkywayathome_client_gb300 import sharding
    for total in (0, 1, 7, 100, 1001, 2800, 10 ** 6 + 3):
        for n in (1, 2, 3, 7, 16):
            b = [sharding.slice_bounds(total, r, n) for r in range(n)]
            assert b[0][0] == 0 and b[-1][1] == total
            assert all(b[i][1] == b[i + 1][0] for i in range(n - 1))
    with pytest.raises(ValueError):
        sharding.slice_bounds(10, 2, 2)


def test_compensated_sum_is_order_exact():
    from milkywayathome_client_gb300 import sharding
    rows = np.array([[1e16], [1.0], [-1e16], [1.0]])
    assert sharding.compensated_sum(rows)[0] == 2.0
    assert sharding.likelihood_compose([[-100.0, 0.0], [-50.0, 0.0]], 50) == -6.0
