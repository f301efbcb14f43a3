"""Host-side logic of the learned outer-iteration accelerator (no GPU)."""
import numpy as np

from staticbtesolver_gb300 import learned


def test_jump_rows_replays_the_solver_rule():
    # every jump pays off: a jump every EVERY iterations from iteration 3 on
    m = 10.0 * 0.8 ** np.arange(40)
    good = m.copy()
    for j in range(3, 40, 6):
        good[j + 1:] *= 0.1
    jumps, reverts = learned.jump_rows(good, 6, tol=0.0)
    assert jumps == [3, 9, 15, 21, 27, 33, 39] and reverts == []
    # the margin 5 iterations after the jump at 3 is not below the margin at
    # the jump: restore, and no more jumps
    bad = m.copy()
    bad[8] = bad[3]
    jumps, reverts = learned.jump_rows(bad, 6, tol=0.0)
    assert jumps == [3] and reverts == [8]
    # no jump on or after the converged iteration
    g2 = good.copy()
    g2[12] = 1e-6
    assert learned.jump_rows(g2, 6, tol=1e-5) == ([3, 9], [])


def test_windows_spanning_a_jump_are_skipped():
    n = 5
    hist = np.cumsum(np.ones((12, n)), axis=0) * 0.01 + 300.0
    fg = dict(centroid=np.zeros((n, 3)), volume=np.ones(n), vmean=1.0, xmin=0.0, xspan=1.0, ymin=0.0, yspan=1.0,
              kn_num=1.0, inv_dim=0.5)
    X, Y = learned.samples_from_history(hist, fg, every=1, jumps=[5])
    # windows k = 3..10; those with a jump at 5 in [k-3, k-1] (k = 6, 7, 8) are dropped
    assert len(Y) == (8 - 3) * n


def test_mirrored_features_flip_sign():
    X = np.arange(16, dtype=np.float32).reshape(2, 8)
    Y = np.array([1.0, -2.0], np.float32)
    Xm, Ym = learned.mirrored(X, Y)
    assert np.array_equal(Xm[2:, :4], -X[:, :4]) and np.array_equal(Xm[2:, 4:], X[:, 4:])
    assert np.array_equal(Ym, [1.0, -2.0, -1.0, 2.0])


def test_scaled_touches_only_the_output_layer():
    p = learned.init_params(3)
    q = learned.scaled(p, 0.0)
    assert np.array_equal(q[: learned.NPARAM - 129], p[: learned.NPARAM - 129])
    assert not q[learned.NPARAM - 129:].any()
