"""Replicas on CPU: frame partition, TwoSum state merge, and the gather +
merge over a world_size-2 gloo process group, including a rank that dies
before the collective (the survivor must get an error, not a partial merge).
No GPU: the merge is host code and the states are built on the host."""
import multiprocessing as mp
import os
import socket
import time

import numpy as np
import pytest

from serstacker_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _state_from_sums(S, W):
    """compensated f32 state (4, h, w) of exact FP64 sums"""
    s32 = S.astype(np.float32)
    w32 = W.astype(np.float32)
    return np.stack([s32, (S - s32).astype(np.float32), w32, (W - w32).astype(np.float32)])


def _partial(frames, weights, lo, hi):
    S = np.zeros(frames.shape[1:])
    W = np.zeros(frames.shape[1:])
    for f in range(lo, hi):
        S += weights[f] * frames[f]
        W += weights[f]
    return S, W


def _data(n=10, h=6, w=7, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 1, size=(n, h, w)), rng.uniform(0.5, 2.0, size=n)


def test_frame_range_partitions_contiguously():
    for n in (0, 1, 7, 2000):
        for world in (1, 2, 3, 8):
            spans = [replicas.frame_range(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c and a <= b
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.frame_range(5, 2, 2)


def test_merge_is_error_free_in_the_leading_sums():
    rng = np.random.default_rng(3)
    a = rng.uniform(-1e4, 1e4, size=(4, 5, 6)).astype(np.float32)
    b = rng.uniform(-1e-3, 1e-3, size=(4, 5, 6)).astype(np.float32)
    a[1], a[3] = a[1] * 1e-8, a[3] * 1e-8          # compensations are small
    m = replicas.merge_states([a, b])
    for k in (0, 2):
        exact = (a[k].astype(np.float64) + a[k + 1]) + (b[k].astype(np.float64) + b[k + 1])
        got = m[k].astype(np.float64) + m[k + 1]
        assert np.abs(got - exact).max() <= 1e-12 * np.abs(exact).max()
    # Bayer states: three groups of four planes
    g = rng.uniform(0, 1, size=(3, 4, 5, 6)).astype(np.float32)
    m3 = replicas.merge_states([g, g])
    assert np.allclose(m3[:, 0].astype(np.float64) + m3[:, 1], 2 * (g[:, 0].astype(np.float64) + g[:, 1]),
                       rtol=1e-12, atol=0)


def test_merge_matches_single_process_sums():
    frames, weights = _data()
    n = len(weights)
    parts = [_state_from_sums(*_partial(frames, weights, *replicas.frame_range(n, 3, r))) for r in range(3)]
    m = replicas.merge_states(parts)
    S, W = _partial(frames, weights, 0, n)
    assert np.abs((m[0].astype(np.float64) + m[1]) - S).max() <= 1e-12 * S.max()
    assert np.abs((m[2].astype(np.float64) + m[3]) - W).max() <= 1e-12 * W.max()
    assert np.array_equal(m, replicas.merge_states(parts))        # fixed order: same planes every run


def _worker(rank, world, port, die_rank, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime

    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
        frames, weights = _data()
        lo, hi = replicas.frame_range(len(weights), world, rank)
        state = _state_from_sums(*_partial(frames, weights, lo, hi))
        if rank == die_rank:
            os._exit(3)                                  # dies between steps, before the collective
        t0 = time.time()
        merged, total = replicas.gather_and_merge(state, hi - lo)
        q.put((rank, "ok", merged, total, time.time() - t0))
        dist.destroy_process_group()
    except Exception as e:                               # the survivor reports the failure
        q.put((rank, "error", repr(e), None, None))


def _run(world, die_rank):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, die_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    expected = world if die_rank < 0 else world - 1
    out = []
    deadline = time.time() + 120
    while len(out) < expected and time.time() < deadline:
        try:
            out.append(q.get(timeout=5))
        except Exception:
            pass
    for p in procs:
        p.join(timeout=30)
        if p.is_alive():
            p.kill()
            p.join()
    return out, [p.exitcode for p in procs]


def test_gloo_two_ranks_merge():
    out, codes = _run(2, -1)
    assert len(out) == 2 and all(o[1] == "ok" for o in out), out
    assert codes == [0, 0]
    frames, weights = _data()
    S, W = _partial(frames, weights, 0, len(weights))
    (_, _, m0, t0, _), (_, _, m1, t1, _) = sorted(out, key=lambda o: o[0])
    assert np.array_equal(m0, m1) and t0 == t1 == len(weights)
    assert np.abs((m0[0].astype(np.float64) + m0[1]) - S).max() <= 1e-12 * S.max()
    assert np.abs((m0[2].astype(np.float64) + m0[3]) - W).max() <= 1e-12 * W.max()


def test_gloo_rank_failure_is_reported():
    out, codes = _run(2, 1)
    assert codes[1] == 3
    assert len(out) == 1 and out[0][0] == 0
    assert out[0][1] == "error", out
