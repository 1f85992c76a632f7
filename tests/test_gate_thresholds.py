"""The MIXED team kernel takes the reference's FP64 gate decisions (core/sim/Integrator.cpp:676-699
for the displacement gate, :725-741 for the residual gate) on FP32 maxima g by comparing g with FP32
thresholds: (double)g ≤ T exactly when g ≤ T rounded toward −∞, and (double)g / scale ≤ relTol
exactly when g ≤ the largest float passing that test (found once per substep by stepping from
relTol·scale rounded down). These checks restate that rule in numpy and compare it with the FP64
decision itself on random and adversarial values (no GPU)."""
import numpy as np

F32 = np.float32


def round_down(t: float) -> np.float32:
    """t rounded toward −∞ to a float (what __double2float_rd does for finite t)."""
    f = F32(t)
    if float(f) > t:
        f = np.nextafter(f, F32(-np.inf))
    return f


def rel_threshold(rel_tol: float, scale: float) -> np.float32:
    """The largest float g with (double)g / scale ≤ rel_tol (scale > 0, rel_tol > 0)."""
    passes = lambda g: float(g) / scale <= rel_tol
    t = round_down(rel_tol * scale)
    for _ in range(64):
        if passes(t) or t == -np.inf:
            break
        t = np.nextafter(t, F32(-np.inf))
    for _ in range(64):
        up = np.nextafter(t, F32(np.inf))
        if t == np.inf or not passes(up):
            break
        t = up
    return t


def test_round_down_threshold_is_exact():
    rng = np.random.default_rng(7)
    for _ in range(2000):
        T = float(10.0 ** rng.uniform(-12, 3))
        thr = round_down(T)
        near = [thr, np.nextafter(thr, F32(np.inf)), np.nextafter(thr, F32(-np.inf)), F32(T), F32(0.0)]
        for g in near + [F32(x) for x in rng.uniform(0, 2 * T, 8)]:
            assert (float(g) <= T) == (g <= thr)


def test_relative_threshold_is_exact():
    rng = np.random.default_rng(11)
    for _ in range(2000):
        rel_tol = float(10.0 ** rng.uniform(-9, -1))
        scale = float(10.0 ** rng.uniform(-8, 1))
        thr = rel_threshold(rel_tol, scale)
        cands = [thr, np.nextafter(thr, F32(np.inf)), np.nextafter(thr, F32(-np.inf)), F32(rel_tol * scale)]
        cands += [F32(x) for x in rng.uniform(0, 3 * rel_tol * scale, 8)]
        for g in cands:
            assert (float(g) / scale <= rel_tol) == (g <= thr)


def test_nan_never_passes():
    g = F32(np.nan)
    assert not (g <= round_down(1e-3)) and not (float(g) <= 1e-3)
    assert not (g <= rel_threshold(1e-3, 2.0))
