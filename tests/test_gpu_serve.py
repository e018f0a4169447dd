"""The request server (continuous batching): results in a mixed, batched stream are the same
as the same requests run one at a time, builds equal the oracle, rebalances rebuild with the
reference's rule, and admission waits for memory."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_stream(engine, oracle, requests, one_at_a_time: bool):
    """requests: list of ("build", kind, seed, n, d) | ("gen", kind, seed, n, d) |
    ("rebalance", build_index, seed, sigma). Returns {build index: fetched results}."""
    opts = dict(hbm_budget_bytes=1 << 30)
    if one_at_a_time:
        opts.update(max_batch=1, lanes=1)
    inst = {}
    with engine.Server(0, **opts) as sv:
        rids = []
        for i, r in enumerate(requests):
            if r[0] == "build":
                _, kind, seed, n, d = r
                gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
                x, y, z = gen(seed, n)
                rid = sv.submit_build(x, y, z, d)
                inst[i] = rid
            elif r[0] == "gen":
                _, kind, seed, n, d = r
                k = engine.ORB_GEN_UNIFORM if kind == "uniform" else engine.ORB_GEN_PLUMMER
                rid = sv.submit_generate(k, seed, n, d)
                inst[i] = rid
            else:
                _, target, seed, sigma = r
                rid = sv.submit_rebalance(inst[target], seed, sigma)
            rids.append(rid)
            if one_at_a_time:
                assert sv.wait(rid)["status"] == 0
        results = [sv.wait(rid) for rid in rids]
        assert all(r["status"] == 0 for r in results)
        fetched = {i: sv.fetch(rid) for i, rid in inst.items()}
        stats = sv.stats()
    return fetched, results, stats


def mixed_requests():
    reqs = [("build", "uniform", 11, 30000, 64), ("gen", "plummer", 12, 50000, 256),
            ("build", "plummer", 13, 8000, 16), ("gen", "uniform", 14, 120000, 1024)]
    reqs += [("rebalance", 0, 100, 1e-3), ("rebalance", 1, 101, 1e-3),
             ("build", "uniform", 15, 200, 8), ("rebalance", 0, 102, 5e-3),
             ("rebalance", 3, 103, 1e-3), ("gen", "uniform", 16, 70000, 128),
             ("rebalance", 2, 104, 2e-2), ("rebalance", 9, 105, 1e-3)]
    return reqs


def test_mix_equals_one_at_a_time(engine, oracle):
    reqs = mixed_requests()
    mixed, res_m, stats = run_stream(engine, oracle, reqs, one_at_a_time=False)
    alone, _, _ = run_stream(engine, oracle, reqs, one_at_a_time=True)
    assert stats["batches"] < len(reqs)  # requests were batched together
    for i in mixed:
        for a, b in zip(mixed[i], alone[i]):
            assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8)), \
                f"instance of request {i} differs between the mix and one at a time"


def test_server_builds_equal_oracle(engine, oracle):
    reqs = [("build", "uniform", 21, 40000, 128), ("build", "plummer", 22, 25000, 64)]
    fetched, _, _ = run_stream(engine, oracle, reqs, one_at_a_time=False)
    for i, (_, kind, seed, n, d) in enumerate(reqs):
        gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
        ref = oracle.build_tree(*gen(seed, n), d)
        heap, ranges, x, y, z, ident = fetched[i]
        assert heap.tobytes() == ref.heap.tobytes()
        assert np.array_equal(ranges, ref.ranges[0])
        assert np.array_equal(ident, ref.perm)
        assert np.array_equal(x.view(np.uint32), ref.x.view(np.uint32))


def test_rebalance_rebuilds_displaced_particles(engine, oracle):
    n, d = 30000, 128
    x, y, z = oracle.gen_uniform(31, n)
    with engine.Server(0, hbm_budget_bytes=1 << 28) as sv:
        inst = sv.submit_build(x, y, z, d)
        sv.wait(inst)
        _, _, x0, y0, z0, id0 = sv.fetch(inst)
        sv.wait(sv.submit_rebalance(inst, 7, 1e-3))
        heap, ranges, x1, y1, z1, id1 = sv.fetch(inst)
    # the rebuild's permutation: position p now holds the particle that sat at perm[p]
    where = np.empty(n, np.int64)
    where[id0] = np.arange(n)
    perm = where[id1]
    pre = [np.empty(n, np.float32) for _ in range(3)]
    for a, post in zip(pre, (x1, y1, z1)):
        a[perm] = post
    # small displacements, inside the box
    disp = np.abs(pre[0].astype(np.float64) - x0)
    assert disp.max() < 1e-2 and disp.mean() > 1e-4
    for a in pre:
        assert a.min() >= -0.5 and a.max() < 0.5
    ref = oracle.build_tree(pre[0], pre[1], pre[2], d)
    assert heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(ranges, ref.ranges[0])
    assert np.array_equal(x1.view(np.uint32), ref.x.view(np.uint32))


def test_admission_waits_for_memory(engine, oracle):
    # arena of ~2.9M particles: the second instance only fits after the first is released
    with engine.Server(0, hbm_budget_bytes=100 << 20, lanes=2) as sv:
        cap = sv.stats()["arena_particles"]
        big = int(cap * 0.7)
        a = sv.submit_generate(engine.ORB_GEN_UNIFORM, 1, big, 64)
        assert sv.wait(a)["status"] == 0
        b = sv.submit_generate(engine.ORB_GEN_UNIFORM, 2, big, 64)
        time.sleep(0.5)
        st = sv.stats()
        assert st["pending"] == 1 and st["requests_done"] == 1
        sv.release(a)
        assert sv.wait(b)["status"] == 0
        # a request larger than the whole arena is refused at submission
        with pytest.raises(engine.OrbError):
            sv.submit_generate(engine.ORB_GEN_UNIFORM, 3, cap + 1, 64)
