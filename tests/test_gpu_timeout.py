"""Failure detection without a GPU fault: a bounded device wait that runs out.

The partition's tile scan chains its blocks with a decoupled look-back, each wait bounded
(orb_test_set_scan_wait sets the bound). Starting the scan's block ticket at 1 leaves the
first status slot unpublished, so the next block's wait can only end by giving up. It must
give up within its bound, flag the build (the kernels that read the scan's prefixes then do
nothing) and orb_build must return ORB_ERR_TIMEOUT; the same context must then build the
oracle's tree bit for bit. The reference has no such path: its errors end the process
(src/constants.h:19-23)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORB_ERR_TIMEOUT = 6


@pytest.fixture
def fresh(engine):
    c = engine.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("spin_limit", [256, 4096])
def test_lookback_wait_gives_up_and_context_recovers(fresh, engine, oracle, spin_limit):
    # 2^23 particles: the root level has 2048 partition tiles, three scan blocks, so the
    # second block's look-back waits on the slot no block takes
    n, d = 1 << 23, 4
    x, y, z = oracle.gen_uniform(606, n)
    fresh.test_set_scan_wait(spin_limit, 1)
    with pytest.raises(engine.OrbError) as e:
        fresh.build(x.copy(), y.copy(), z.copy(), d)
    assert e.value.status == ORB_ERR_TIMEOUT
    fresh.test_set_scan_wait(0, 0)
    ref = oracle.build_tree(x, y, z, d)
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    res = fresh.build(gx, gy, gz, d)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    assert np.array_equal(res.perm, ref.perm)
    assert np.array_equal(gx.view(np.uint32), ref.x.view(np.uint32))


def test_lookback_timeout_in_a_batch_and_service_call(fresh, engine, oracle):
    """The same bounded wait in a batched build and in the service partition."""
    n = 1 << 23
    x, y, z = oracle.gen_uniform(607, n)
    fresh.test_set_scan_wait(512, 1)
    with pytest.raises(engine.OrbError) as e:
        fresh.build_batch(x.copy(), y.copy(), z.copy(), [{"offset": 0, "n": n, "d": 2}])
    assert e.value.status == ORB_ERR_TIMEOUT
    fresh.load_particles(x, y, z, 3)
    root = np.zeros(1, engine.CELL_DTYPE)
    root["nLeafCells"], root["cutAxis"], root["prevCutAxis"] = 2, 0, -1
    root["cutMarginLeft"], root["cutMarginRight"] = -0.5, 0.5
    with pytest.raises(engine.OrbError) as e:
        fresh.partition(root)
    assert e.value.status == ORB_ERR_TIMEOUT
    fresh.test_set_scan_wait(0, 0)
    with pytest.raises(engine.OrbError):
        fresh.test_set_scan_wait(0, 256)  # the ticket hook takes one byte
    parts, perm, _ = fresh.build_batch(x.copy(), y.copy(), z.copy(), [{"offset": 0, "n": n, "d": 2}])
    ref = oracle.build_tree(x, y, z, 2)
    assert parts[0][0].tobytes() == ref.heap.tobytes()
    assert np.array_equal(perm, ref.perm)
