"""The MIXED team kernel reduces each product warp's 33 partial sums (11 rows × 3 components of
Ã⁻¹·r) over its 32 lanes with a transposing shuffle reduction: at the step with offset O, a lane
with bit O set keeps the upper half of its first 2·O values and sends the lower half to its
partner (lane ^ O), the other lane the reverse, and each adds what it receives. After the steps
16, 8, 4, 2, 1, lane l holds the warp's sum of value l; the 33rd value is summed by a plain
butterfly. This emulates those shuffles lane by lane in numpy and checks the mapping the kernel
writes out with (out[l] = value l for l < 3·rows, out[32] = value 32), in the kernel's order of
additions, against a sum taken in float64 (no GPU)."""
import numpy as np


def transpose_reduce(vals: np.ndarray) -> np.ndarray:
    """vals: (32 lanes, 32 values) float32 → (32,) lane l's result after the five steps."""
    s = vals.astype(np.float32).copy()
    lanes = np.arange(32)
    for o in (16, 8, 4, 2, 1):
        up = (lanes & o) != 0
        send = np.where(up[:, None], s[:, :o], s[:, o:2 * o])
        keep = np.where(up[:, None], s[:, o:2 * o], s[:, :o])
        recv = send[lanes ^ o]  # __shfl_xor_sync(send, o)
        s[:, :o] = keep + recv
    return s[:, 0]


def butterfly(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.float32).copy()
    lanes = np.arange(32)
    for o in (16, 8, 4, 2, 1):
        v = v + v[lanes ^ o]
    return v


def test_lane_l_holds_the_sum_of_value_l():
    rng = np.random.default_rng(3)
    for _ in range(50):
        vals = rng.standard_normal((32, 33)).astype(np.float32)
        got = transpose_reduce(vals[:, :32])
        want = vals[:, :32].astype(np.float64).sum(axis=0)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-5 * np.abs(vals).sum(axis=0)[:32].max())
        last = butterfly(vals[:, 32])
        assert np.all(last == last[0])  # every lane ends with the same 33rd sum
        np.testing.assert_allclose(last[0], vals[:, 32].astype(np.float64).sum(), rtol=1e-5, atol=1e-5)


def test_exact_on_integers():
    # small integers add exactly in float32, so the mapping is checked without rounding
    rng = np.random.default_rng(5)
    vals = rng.integers(-1000, 1000, size=(32, 32)).astype(np.float32)
    got = transpose_reduce(vals)
    assert np.array_equal(got, vals.sum(axis=0))
