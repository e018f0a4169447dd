"""The sampled first count pass (k_sample + the predicted mode of the count pass), against the
oracle bit for bit.

The first count pass of a cell of at least 2^18 particles bins only the keys of a bracket
predicted from a strided sample of the cell; the exact counts below and above the bracket
decide whether the replay of the reference loop may use it, and the pass is repeated over
every key when they do not. Results must not depend on the prediction: the tests compare
with the oracle under the default width, under a width of one standard error (many
misses, so the fallback runs) and with the prediction off."""
import numpy as np
import pytest

from test_gpu_batch import check_batch
from test_gpu_parity import run_both

pytestmark = pytest.mark.gpu


@pytest.fixture()
def tuned(ctx):
    """The session context, its tuning restored after the test."""
    saved = ctx.get_tuning()
    yield ctx
    ctx.set_tuning(**saved)


@pytest.mark.parametrize("sigmas", [5, 1, 0])
def test_sampled_uniform_matches_oracle(tuned, oracle, sigmas):
    tuned.set_tuning(predict_sigmas=sigmas)
    x, y, z = oracle.gen_uniform(77, 1 << 22)
    res, _ = run_both(tuned, oracle, x, y, z, 1 << 8)
    info = res.info
    if sigmas == 0:
        assert info["sampled_cells"] == 0
    else:
        # levels 0..3 hold cells of 2^22..2^19 particles (15 cells, all sampled); level 4
        # cells of 2^18 +- 2 (sampled from 2^18 up)
        assert 15 <= info["sampled_cells"] <= 31
    if sigmas == 1:
        # a bracket of one standard error each side misses about a third of the time
        assert info["sampled_misses"] > 0
    if sigmas == 5:
        assert info["sampled_misses"] <= 1


def test_sampled_plummer_matches_oracle(tuned, oracle):
    x, y, z = oracle.gen_plummer(78, (1 << 22) + 999)
    for sigmas in (5, 2):
        tuned.set_tuning(predict_sigmas=sigmas)
        res, _ = run_both(tuned, oracle, x, y, z, 1 << 10)
        assert res.info["sampled_cells"] > 0


def test_sampled_sorted_and_tied_keys(tuned, oracle):
    """Cells whose keys are sorted along the cut axis (strided samples are exact quantiles)
    and cells whose keys take 256 values (brackets of one value, cuts on keys)."""
    rng = np.random.default_rng(79)
    n = 1 << 21
    x = np.sort(rng.random(n, dtype=np.float32) - np.float32(0.5))
    y = rng.random(n, dtype=np.float32) - np.float32(0.5)
    z = rng.random(n, dtype=np.float32) - np.float32(0.5)
    for sigmas in (5, 1):
        tuned.set_tuning(predict_sigmas=sigmas)
        res, _ = run_both(tuned, oracle, x, y, z, 1 << 6)
        assert res.info["sampled_cells"] > 0
    g = [(rng.integers(0, 256, n).astype(np.float32) / np.float32(256) - np.float32(0.5))
         for _ in range(3)]
    for sigmas in (5, 1):
        tuned.set_tuning(predict_sigmas=sigmas)
        run_both(tuned, oracle, *g, 1 << 6)


def test_sampled_batch_matches_oracle(tuned, oracle):
    """Batched instances large enough for sampled passes next to small ones."""
    specs = [("uniform", 80, (1 << 20) + 7, 1 << 6, 0), ("plummer", 81, 1 << 19, 1 << 8, 0),
             ("uniform", 82, 5000, 1 << 4, 0), ("plummer", 83, (1 << 18) + 3, 1 << 5, 0)]
    for sigmas in (5, 1):
        tuned.set_tuning(predict_sigmas=sigmas)
        _, info = check_batch(tuned, oracle, specs)
        assert info["sampled_cells"] > 0
