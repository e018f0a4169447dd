"""The largest build the ABI accepts: n = 2^31 - 1 particles (positions, counts and the
permutation are 32-bit) into 2^21 leaves, compared bit for bit with the oracle (heap, ranges,
permutation, coordinates). About 24 GB of particles on the device and 70 GB of host memory for
the check; skipped where either is not available."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N_MAX = (1 << 31) - 1
D = 1 << 21


def host_bytes():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_AVPHYS_PAGES")
    except (ValueError, OSError):
        return 0


def test_max_particles_bit_exact(ctx, oracle, engine):
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    free, _ = torch.cuda.mem_get_info()
    if free < (80 << 30) or host_bytes() < (100 << 30):
        pytest.skip("needs 80 GB of free device memory and 100 GB of host memory")
    n, d = N_MAX, D
    x, y, z = (torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3))
    ctx.generate(engine.ORB_GEN_UNIFORM, 2026, n, x, y, z, device_pointers=True)
    torch.cuda.synchronize()
    hx, hy, hz = (a.cpu().numpy() for a in (x, y, z))  # the inputs, for the oracle
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    res = ctx.build(x, y, z, d, perm=perm, device_pointers=True)
    assert res.info["levels_built"] == 21
    gx, gy, gz = (a.cpu().numpy() for a in (x, y, z))
    gperm = perm.cpu().numpy().view(np.uint32)
    del x, y, z, perm
    torch.cuda.empty_cache()
    ref = oracle.build_tree(hx, hy, hz, d, copy=False, threads=os.cpu_count() or 1)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    assert np.array_equal(gperm, ref.perm)
    for got, want in ((gx, ref.x), (gy, ref.y), (gz, ref.z)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the leaves tile [0, n) in heap order
    leaf = res.ranges[d - 1:].astype(np.int64)
    assert leaf[0, 0] == 0 and leaf[-1, 1] == n and np.array_equal(leaf[1:, 0], leaf[:-1, 1])
