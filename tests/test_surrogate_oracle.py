"""The CPU oracle of the learned far field, pinned without a GPU: its backward
pass against central finite differences, its targets against a direct loop
over the reference's medium-distance formula (sim_kernels.cl:940-955), and
the linearity the network is built on."""
import numpy as np

from oracle import surrogate_ref as S


def _weights(rng, scale=0.2):
    w = []
    for ci, co, _ in S.LAYERS:
        w.append(rng.normal(0.0, scale / np.sqrt(ci * 27), ci * co * 27))
    return np.concatenate(w)


def test_weight_count():
    assert S.weight_count() == (4 * 32 + 8 * 32 * 32 + 32 * 168) * 27


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    nd = 4
    w = _weights(rng, 1.0)
    x = rng.uniform(-1, 1, (2, 4, nd ** 3))
    t = rng.normal(0, 1, (2, S.OUT_PAD, nd ** 3))
    loss, g = S.loss_and_grad(w, x, t)
    assert np.isfinite(loss)
    offs = np.cumsum([0] + [ci * co * 27 for ci, co, _ in S.LAYERS])
    idx = np.concatenate([rng.integers(offs[l], offs[l + 1], 4) for l in range(10)])
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (S.loss_and_grad(wp, x, t)[0] - S.loss_and_grad(wm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def test_forward_is_linear():
    rng = np.random.default_rng(8)
    w = _weights(rng)
    x1 = rng.uniform(-1, 1, (1, 4, 64))
    x2 = rng.uniform(-1, 1, (1, 4, 64))
    y = S.forward(w, 2.5 * x1 - 0.5 * x2)
    assert np.allclose(y, 2.5 * S.forward(w, x1) - 0.5 * S.forward(w, x2), rtol=1e-12, atol=1e-12)


def test_targets_match_direct_loop():
    """Bins farther than RNEAR from the block, summed one by one with the
    reference's vec_r / |vec_r|^3 form at each corner cell."""
    rng = np.random.default_rng(9)
    nd, bs = 4, (6.0, 5.0, 4.0)
    V = nd ** 3
    x = rng.uniform(-1, 1, (1, 4, V))
    t = S.far_targets(x, nd, bs, rnear=1)
    assert not t[:, S.OUT_CH:].any()
    for v in (0, 21, 63):
        bx, by, bz = v % nd, (v // nd) % nd, v // (nd * nd)
        for c in (0, 5, 13, 26):
            p = np.array([bx * bs[0] + 0.5 * (c % 3) * (bs[0] - 1), by * bs[1] + 0.5 * ((c // 3) % 3) * (bs[1] - 1),
                          bz * bs[2] + 0.5 * (c // 9) * (bs[2] - 1)])
            e, b = np.zeros(3), np.zeros(3)
            for d in range(V):
                dx, dy, dz = d % nd, (d // nd) % nd, d // (nd * nd)
                if max(abs(dx - bx), abs(dy - by), abs(dz - bz)) <= 1:
                    continue
                r = p - np.array([(dx + 0.5) * bs[0], (dy + 0.5) * bs[1], (dz + 0.5) * bs[2]])
                pre = r / np.linalg.norm(r) ** 3
                e += x[0, 0, d] * pre
                b += np.cross(x[0, 1:, d], pre)
            assert np.allclose(t[0, c * 6:c * 6 + 3, v], e, rtol=1e-12, atol=1e-14)
            assert np.allclose(t[0, c * 6 + 3:c * 6 + 6, v], b, rtol=1e-12, atol=1e-14)


def test_quadratic_weights_reproduce_quadratics():
    for t in (0.0, 0.2, 0.5, 0.77, 1.0):
        w = S.quad_weights(t)
        nodes = np.array([0.0, 0.5, 1.0])
        for f in (lambda u: 1 + 0 * u, lambda u: u, lambda u: 3 * u * u - u + 2):
            assert abs(w @ f(nodes) - f(t)) < 1e-12


def test_near_radius_matches_the_library():
    """The oracle's near radius (which the GPU targets are checked against) is the
    one the Python mirror reports and bench.py counts near terms with."""
    from ionsolver_gb300 import Lbm
    assert S.RNEAR == Lbm.SURROGATE_NEAR_RADIUS
