"""Host-side logic of the serving loop (no GPU): request generation, the
least-recently-used residency policy under a byte budget, continuous
batching, latency percentiles, catalog scene sizes."""
import collections
import math

import numpy as np
import pytest

import __graft_entry__ as graft


@pytest.fixture(scope="module")
def server():
    graft.load_package()
    from habitat_sim_gb300 import server
    return server


def test_random_requests_are_seeded_and_poisson(server):
    cat = server.SceneCatalog(16, seed=3, tri_range=(1e3, 1e4))
    a = server.random_requests(cat, 2000, rate=500.0, seed=5)
    b = server.random_requests(cat, 2000, rate=500.0, seed=5)
    assert [q.scene for q in a] == [q.scene for q in b]
    assert all(np.array_equal(x.view, y.view) for x, y in zip(a, b))
    arr = np.array([q.arrival for q in a])
    assert (np.diff(arr) >= 0).all()
    gaps = np.diff(np.concatenate([[0.0], arr]))
    assert abs(gaps.mean() - 1 / 500.0) < 0.1 / 500.0      # exponential gaps, mean 1/rate
    res = collections.Counter(q.resolution for q in a)
    assert set(res) <= set(server.CLASSES)
    assert abs(res[128] / 2000 - 0.5) < 0.05
    assert {q.scene for q in a} == set(range(16))


def test_pose_view_is_a_rigid_inverse(server):
    v = server.pose_view(1.0, 1.5, -2.0, 0.3, -0.2, 0.1)
    m = v.T.astype(np.float64)                      # row-major world -> camera
    r = m[:3, :3]
    assert np.allclose(r @ r.T, np.eye(3), atol=1e-6)
    assert np.allclose(m @ np.array([1.0, 1.5, -2.0, 1.0]), [0, 0, 0, 1], atol=1e-6)


def test_residency_evicts_least_recently_used(server):
    res = server.Residency(budget_bytes=100, capacity=3)
    for s, b in [(10, 40), (11, 30), (12, 20)]:
        assert res.plan(b, pinned=set()) == []
        res.add(s, b)
    assert res.touch(10) is not None            # 10 is now the most recent
    # 50 more bytes: 90 + 50 > 100 and no free slot -> evict 11 (oldest), then 12.
    assert res.plan(50, pinned=set()) == [11, 12]
    # With 11 pinned the oldest unpinned go first.
    assert res.plan(50, pinned={11}) == [12, 10]
    for s in res.plan(50, pinned=set()):
        res.remove(s)
    slot = res.add(13, 50)
    assert res.bytes == 90 and list(res.lru) == [10, 13] and 0 <= slot < 3
    with pytest.raises(MemoryError):
        res.plan(101, pinned=set())
    with pytest.raises(MemoryError):
        res.plan(80, pinned={10, 13})


def test_residency_slot_limit(server):
    res = server.Residency(budget_bytes=1 << 40, capacity=2)
    res.add(1, 5)
    res.add(2, 5)
    assert res.plan(5, pinned=set()) == [1]
    slots = {res.remove(1)}
    assert res.add(3, 5) in slots


def test_take_batch_is_fifo_per_class(server):
    q = {64: collections.deque(range(10)), 128: collections.deque(range(100, 103)),
         256: collections.deque()}
    b = server.take_batch(q, {64: 4, 128: 8, 256: 2})
    assert b == {64: [0, 1, 2, 3], 128: [100, 101, 102]}
    assert list(q[64]) == [4, 5, 6, 7, 8, 9] and not q[128]


def test_percentiles(server):
    p = server.percentiles(np.arange(1, 101) / 1000.0)
    assert math.isclose(p["p50_ms"], 50.5) and math.isclose(p["p99_ms"], 99.01)


def test_catalog_scene_sizes(server):
    cat = server.SceneCatalog(4, seed=1, tri_range=(1e4, 1e5))
    for s in range(4):
        a = cat.asset(s)
        assert 0.6 * cat.targets[s] < a.triangles < 1.6 * cat.targets[s]
        assert a.indices.max() < len(a.positions)
        assert set(np.unique(a.object_ids)) == set(range(1, 22))
        # One mesh view per object (the shell, 20 boxes), covering the indices in order.
        assert len(a.parts) == 21
        assert sum(n for (_, n, _) in a.parts) == len(a.indices)
        assert [f for (f, _, _) in a.parts] == list(np.cumsum([0] + [n for (_, n, _) in a.parts])[:-1])
        boxes = 0
        for (_, n, _) in a.parts:
            chunks = (n // 3 + 31) // 32
            boxes += chunks + (chunks + 31) // 32
        assert a.device_bytes() == len(a.positions) * 40 + a.triangles * 12 + 64 * 64 * 4 + boxes * 32
    assert cat.asset(2) is cat.asset(2)


def test_textured_catalog_layers_and_sizes(server):
    """The serving benchmark's textured catalog: a scene of T triangles gets
    max(1, round(T / tris_per_layer)) noise layers, windows of one host pool
    (alpha 255), and object k samples layer k % layers."""
    cat = server.SceneCatalog(6, seed=2, tri_range=(1e4, 1e5), texture_side=64, tris_per_layer=12000,
                              pool_bytes=1 << 22)
    for s in range(6):
        a = cat.asset(s)
        L = max(1, int(round(cat.targets[s] / 12000)))
        assert a.texture.shape == (L, 64, 64, 4) and (a.texture[..., 3] == 255).all()
        assert [layer for (_, _, layer) in a.parts] == [k % L for k in range(21)]
        assert a.device_bytes() > a.texture.size
    assert not np.array_equal(cat.asset(0).texture[0], cat.asset(1).texture[0])


def test_take_batch_caps_the_step():
    """max_batch takes the earliest arrivals across classes, within the slots."""
    import collections
    from habitat_sim_gb300 import server as srv
    reqs = [srv.Request(0, c, None, arrival=t) for (c, t) in ((64, 0.3), (128, 0.1), (64, 0.2))]
    queues = {64: collections.deque([reqs[2], reqs[0]]), 128: collections.deque([reqs[1]])}
    b = srv.take_batch(queues, {64: 4, 128: 4}, max_batch=2)
    assert b == {128: [reqs[1]], 64: [reqs[2]]} and list(queues[64]) == [reqs[0]]
