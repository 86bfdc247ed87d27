"""Multi-rank host logic on CPU (gloo, world size 2): the pixel-sharded image gradient sums
each rank's loss and gradient with one all-reduce (kgeo_gb300.image_grad.reduce_loss_grad)
and must equal the single-process result. Each rank's part is computed with the image
kernel's arithmetic built for the host (tests/hostmath), as a GPU rank would with the kernel."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import hmlib

DEG = np.pi / 180


def _grid():
    x = np.linspace(-8, 8, 24)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    return A, B


def _loss_grad(A, B, target):
    mi, md = hmlib.model_arrays(('bpl', {'p1': -2.0, 'p2': 0.0}), ('general', {'fac_subkep': 0.8, 'beta_r': 0.5}))
    I = hmlib.image(0.5, 1.e4, 60 * DEG, A, B, 3, mi, md)['I']
    jac, _ = hmlib.image_jac(0.5, 1.e4, 60 * DEG, A, B, 3, mi, md)
    r = I - target
    return float((r * r).sum()), list(np.einsum('pm,pmq->q', 2 * r, jac))


def _worker(rank, world, port, q):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        from kgeo_gb300.image_grad import reduce_loss_grad
        A, B = _grid()
        target = np.random.default_rng(1).uniform(0, 0.1, (A.size, 3))
        sl = np.array_split(np.arange(A.size), world)[rank]
        L, g = _loss_grad(A[sl], B[sl], target[sl])
        q.put((rank, reduce_loss_grad(L, g)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_sharded_gradient_sum_two_ranks():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    A, B = _grid()
    target = np.random.default_rng(1).uniform(0, 0.1, (A.size, 3))
    L, g = _loss_grad(A, B, target)
    for r in (0, 1):
        Lr, gr = res[r]
        assert abs(Lr - L) <= 1e-12 * abs(L)
        np.testing.assert_allclose(gr, g, rtol=1e-12, atol=1e-14)


def test_reduce_without_process_group_is_identity():
    from kgeo_gb300.image_grad import reduce_loss_grad
    L, g = reduce_loss_grad(1.5, [1.0, -2.0])
    assert L == 1.5 and g == [1.0, -2.0]


def _trace_worker(rank, world, port, q):
    """One rank of the benchmark's multi-GPU split: its contiguous pixel range of the image
    (bench.shard), traced with the kernel arithmetic built for the host; rank 0 gathers."""
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        import sys
        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        import bench
        import test_hostmath_cpu as T
        import ctypes
        L = ctypes.CDLL(T.LIBPATH)
        L.hm_setup.restype = ctypes.c_uint
        a, th_o, A, B = bench.workload(0, grid=20)
        lo, hi = bench.shard(A.size, rank, world)
        part = T.host_trace_stepped(L, a, bench.R_O, th_o, A[lo:hi], B[lo:hi], 40, 16)
        parts = [None] * world
        dist.all_gather_object(parts, (lo, hi, part))
        if rank == 0:
            q.put(parts)
    finally:
        dist.destroy_process_group()


def test_pixel_shards_concatenate_to_single_trace():
    """Rays are independent: the ranks' contiguous pixel ranges, concatenated, are the
    single-process trace of the whole image, sample for sample. Every trace runs in a spawned
    process (world size 1 for the whole image), so all of them load the same host build."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import test_hostmath_cpu as T
    if not os.path.exists(T.LIBPATH):
        import pytest
        pytest.skip('host build of the kernel headers missing')
    results = {}
    for world in (1, 2, 3):
        ctx = mp.get_context('spawn')
        q = ctx.Queue()
        port = _free_port()
        procs = [ctx.Process(target=_trace_worker, args=(r, world, port, q)) for r in range(world)]
        for p in procs:
            p.start()
        results[world] = q.get(timeout=120)
        for p in procs:
            p.join(timeout=60)
            assert p.exitcode == 0
    whole = results[1][0][2]
    npix = results[1][0][1]
    for world in (2, 3):
        parts = results[world]
        assert [p[0] for p in parts] == sorted(p[0] for p in parts) and parts[-1][1] == npix
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
        for k in ('t', 'r', 'th', 'ph', 'sig', 'mino'):
            cat = np.concatenate([p[2][k] for p in parts], axis=1)
            np.testing.assert_array_equal(cat, whole[k])
