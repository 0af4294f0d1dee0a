"""CPU checks that pin the empty-space oracle itself: the proposal network's
analytic gradient against central differences, and the occupancy grid's
definition on a hand-checkable volume."""

import numpy as np

from oracle import empty_space_oracle as eso


def test_proposal_gradient_matches_central_differences():
    rng = np.random.default_rng(0)
    P = rng.standard_normal(8450) * 0.2
    X = rng.standard_normal((7, 64))
    T = rng.uniform(0, 1, (7, 2))
    V = np.array([1, 1, 0, 1, 1, 1, 1], np.uint8)
    loss, g = eso.proposal_loss_grad(P, X, T, V, alpha=5.0, inv_count=1 / 7)
    h = 1e-6
    idx = rng.choice(8450, 60, replace=False).tolist() + [8448, 8449, 0, 4096, 8320]
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        num = (eso.proposal_loss_grad(Pp, X, T, V, 5.0, 1 / 7)[0] - eso.proposal_loss_grad(Pm, X, T, V, 5.0, 1 / 7)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), i


def test_occupancy_grid_definition():
    vol = np.zeros((9, 10, 11), np.float32)
    vol[4, 5, 6] = 1.0
    g = eso.occupancy_grid(vol, cell=2, max_dist=4)
    assert g.shape == (9 // 2 + 1 + 2, 10 // 2 + 2, 11 // 2 + 1 + 2)
    # cell gx covers voxels [(gx - 1) * 2, gx * 2) dilated by 2: voxel 6 is in
    # the dilated range of cells gx with (gx - 1) * 2 - 2 <= 6 <= gx * 2 + 1
    occ_x = [gx for gx in range(g.shape[2]) if (gx - 1) * 2 - 2 <= 6 <= gx * 2 + 1]
    occ = np.argwhere(g == 0)
    assert sorted(set(occ[:, 2].tolist())) == occ_x
    # Chebyshev distances grow by one per cell away from the occupied block
    zc, yc, xc = occ.min(0)
    assert g[zc, yc, max(xc - 1, 0)] in (0, 1)
    assert g.max() <= 4


def test_features_encode_entry_and_exit():
    p0 = np.array([[-5.0, 3.0, 4.0], [1.0, -8.0, 2.0]])
    d = np.array([[20.0, 0.0, 0.0], [0.0, 20.0, 0.5]])
    f, t0, t1, hit = eso.proposal_features(p0, d, (8, 8, 8))
    assert hit.all()
    np.testing.assert_allclose(f[0, :6], [-1 / 8, 3 / 8, 4 / 8, 1.0, 3 / 8, 4 / 8], atol=1e-12)
    np.testing.assert_allclose(f[:, 6:12], np.sin(np.pi * f[:, :6]), atol=1e-12)
    assert (f[:, 54:] == 0).all()
