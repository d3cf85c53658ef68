"""CPU oracle (float64 numpy) of the learned far field.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU
network kernels.  The product path never calls it.

The learned far field has no counterpart in the reference; what it
approximates is the medium-distance loop of update_e_b_dynamic
(IonSolver src/kernels/sim_kernels.cl:940-955): every depth-D LOD bin d in
[NUM_LOD_OWN - 8^D, NUM_LOD_OWN) other than the cell's own bin adds
    E += q_d (r - c_d) / |r - c_d|^3,   B += q_d v_d x (r - c_d) / |r - c_d|^3
with bin centres c_d = (i + 1/2) * block size (lod_coordinates, :436-444).
The network sees the bins on their 8^D grid (index v = x + (y + z nd) nd);
the part it learns is the sum over bins farther than RNEAR (Chebyshev) from
the block, taken at 27 nodes of the block (interpolated triquadratically per
cell).

Contents: the layer table, a 3-D convolution with zero padding and dilation
on the [C][z][y][x] layout, the residual forward pass, its backward pass for
the mean squared error, and the exact targets.
"""
from __future__ import annotations

import numpy as np

RNEAR = 1
NODES = 27           # 3 x 3 x 3 interpolation nodes per block (offsets 0, (bs-1)/2, bs-1 on each axis)
OUT_CH = NODES * 6   # (Ex, Ey, Ez, Bx, By, Bz) per node
OUT_PAD = 168        # head channels (OUT_CH rounded up to 8; the rest have zero targets)
# (input channels, output channels, dilation) of the ten 3^3 convolutions:
# stem, 4 residual blocks of two convolutions, head
LAYERS = [(4, 32, 1), (32, 32, 1), (32, 32, 2), (32, 32, 2), (32, 32, 4), (32, 32, 4), (32, 32, 8), (32, 32, 1),
          (32, 32, 1), (32, OUT_PAD, 1)]


def weight_count() -> int:
    return sum(ci * co * 27 for ci, co, _ in LAYERS)


def split_weights(w: np.ndarray) -> list[np.ndarray]:
    """Flat weight vector -> per layer [Cout][Cin][27] (tap k: dx = k%3-1, dy = k//3%3-1, dz = k//9-1)."""
    out, o = [], 0
    for ci, co, _ in LAYERS:
        n = ci * co * 27
        out.append(np.asarray(w[o:o + n], np.float64).reshape(co, ci, 27))
        o += n
    return out


def _taps():
    return [(k % 3 - 1, (k // 3) % 3 - 1, k // 9 - 1) for k in range(27)]


def _shift(a: np.ndarray, ox: int, oy: int, oz: int) -> np.ndarray:
    """s[..., z, y, x] = a[..., z+oz, y+oy, x+ox], zero outside."""
    nd = a.shape[-1]
    s = np.zeros_like(a)
    def rng(o):
        return (max(0, -o), min(nd, nd - o))
    (x0, x1), (y0, y1), (z0, z1) = rng(ox), rng(oy), rng(oz)
    if x0 < x1 and y0 < y1 and z0 < z1:
        s[..., z0:z1, y0:y1, x0:x1] = a[..., z0 + oz:z1 + oz, y0 + oy:y1 + oy, x0 + ox:x1 + ox]
    return s


def conv(a: np.ndarray, w: np.ndarray, dil: int) -> np.ndarray:
    """a [B][Cin][nd][nd][nd], w [Cout][Cin][27] -> [B][Cout][nd][nd][nd]."""
    B, _, nd = a.shape[0], a.shape[1], a.shape[-1]
    out = np.zeros((B, w.shape[0], nd, nd, nd))
    for k, (ox, oy, oz) in enumerate(_taps()):
        out += np.einsum("oc,bczyx->bozyx", w[:, :, k], _shift(a, dil * ox, dil * oy, dil * oz))
    return out


def conv_wgrad(a: np.ndarray, g: np.ndarray, dil: int) -> np.ndarray:
    """dL/dw of out = conv(a, w) for upstream gradient g."""
    gw = np.zeros((g.shape[1], a.shape[1], 27))
    for k, (ox, oy, oz) in enumerate(_taps()):
        gw[:, :, k] = np.einsum("bozyx,bczyx->oc", g, _shift(a, dil * ox, dil * oy, dil * oz))
    return gw


def conv_dgrad(g: np.ndarray, w: np.ndarray, dil: int) -> np.ndarray:
    """dL/da of out = conv(a, w) for upstream gradient g."""
    B, nd = g.shape[0], g.shape[-1]
    ga = np.zeros((B, w.shape[1], nd, nd, nd))
    for k, (ox, oy, oz) in enumerate(_taps()):
        ga += _shift(np.einsum("oc,bozyx->bczyx", w[:, :, k], g), -dil * ox, -dil * oy, -dil * oz)
    return ga


def _grid(x: np.ndarray, C: int) -> np.ndarray:
    x = np.asarray(x, np.float64)
    V = x.shape[-1]
    nd = round(V ** (1 / 3))
    return x.reshape(-1, C, nd, nd, nd)


def forward(w: np.ndarray, x: np.ndarray, keep: bool = False):
    """x [B][4][V] -> y [B][OUT_PAD][V]; h_{i+1} = h_i + conv_b(conv_a(h_i))."""
    W = split_weights(w)
    a = _grid(x, 4)
    acts = [a]
    h = conv(a, W[0], LAYERS[0][2])
    for i in range(4):
        t = conv(h, W[1 + 2 * i], LAYERS[1 + 2 * i][2])
        acts += [h, t]
        h = h + conv(t, W[2 + 2 * i], LAYERS[2 + 2 * i][2])
    acts.append(h)
    y = conv(h, W[9], LAYERS[9][2])
    y = y.reshape(y.shape[0], OUT_PAD, -1)
    return (y, acts) if keep else y


def loss_and_grad(w: np.ndarray, x: np.ndarray, t: np.ndarray) -> tuple[float, np.ndarray]:
    """Mean squared error over all outputs and its gradient with respect to the flat weights."""
    W = split_weights(w)
    y, acts = forward(w, x, keep=True)
    t = np.asarray(t, np.float64).reshape(y.shape)
    d = y - t
    loss = float(np.mean(d * d))
    gy = (2.0 * d / d.size).reshape(y.shape[0], OUT_PAD, *acts[0].shape[2:])
    gw = [None] * 10
    x0, h4 = acts[0], acts[-1]
    gw[9] = conv_wgrad(h4, gy, LAYERS[9][2])
    gh = conv_dgrad(gy, W[9], LAYERS[9][2])
    for i in range(3, -1, -1):
        hi, ti = acts[1 + 2 * i], acts[2 + 2 * i]
        gw[2 + 2 * i] = conv_wgrad(ti, gh, LAYERS[2 + 2 * i][2])
        gt = conv_dgrad(gh, W[2 + 2 * i], LAYERS[2 + 2 * i][2])
        gw[1 + 2 * i] = conv_wgrad(hi, gt, LAYERS[1 + 2 * i][2])
        gh = gh + conv_dgrad(gt, W[1 + 2 * i], LAYERS[1 + 2 * i][2])
    gw[0] = conv_wgrad(x0, gh, LAYERS[0][2])
    return loss, np.concatenate([g.reshape(-1) for g in gw])


def node_offsets(bs: tuple[float, float, float]) -> np.ndarray:
    """[27][3] cell offsets of the nodes inside a block: (i/2)(bs-1), node = ix + 3 (iy + 3 iz)."""
    n = np.arange(NODES)
    return np.stack([(n % 3) * 0.5 * (bs[0] - 1), ((n // 3) % 3) * 0.5 * (bs[1] - 1), (n // 9) * 0.5 * (bs[2] - 1)], 1)


def quad_weights(t: float) -> np.ndarray:
    """Lagrange weights of the nodes t = 0, 1/2, 1 at t."""
    return np.array([2 * (t - 0.5) * (t - 1), -4 * t * (t - 1), 2 * t * (t - 0.5)])


def far_targets(x: np.ndarray, nd: int, bs: tuple[float, float, float], rnear: int = RNEAR) -> np.ndarray:
    """Exact far field at the 27 nodes of every block: x [S][4][V] -> [S][OUT_PAD][V]
    (channel = node*6 + (Ex,Ey,Ez,Bx,By,Bz); channels >= OUT_CH are zero)."""
    x = np.asarray(x, np.float64)
    S, V = x.shape[0], nd ** 3
    idx = np.arange(V)
    bx, by, bz = idx % nd, (idx // nd) % nd, idx // (nd * nd)
    cen = np.stack([(bx + 0.5) * bs[0], (by + 0.5) * bs[1], (bz + 0.5) * bs[2]], 1)
    cheb = np.maximum(np.maximum(abs(bx[:, None] - bx[None]), abs(by[:, None] - by[None])), abs(bz[:, None] - bz[None]))
    far = cheb > rnear
    out = np.zeros((S, OUT_PAD, V))
    offs = node_offsets(bs)
    for c in range(NODES):
        p = np.stack([bx * bs[0] + offs[c, 0], by * bs[1] + offs[c, 1], bz * bs[2] + offs[c, 2]], 1)
        R = p[:, None, :] - cen[None, :, :]  # [V target][V source][3]
        r2 = np.sum(R * R, -1)
        inv3 = np.where(far, 1.0 / (r2 * np.sqrt(np.where(far, r2, 1.0))), 0.0)
        q, qx, qy, qz = x[:, 0], x[:, 1], x[:, 2], x[:, 3]  # [S][V]
        Rx, Ry, Rz = R[..., 0] * inv3, R[..., 1] * inv3, R[..., 2] * inv3
        out[:, c * 6 + 0] = q @ Rx.T
        out[:, c * 6 + 1] = q @ Ry.T
        out[:, c * 6 + 2] = q @ Rz.T
        out[:, c * 6 + 3] = qy @ Rz.T - qz @ Ry.T
        out[:, c * 6 + 4] = qz @ Rx.T - qx @ Rz.T
        out[:, c * 6 + 5] = qx @ Ry.T - qy @ Rx.T
    return out
