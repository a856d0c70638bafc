"""The identities behind the folded field (f16x3 on grids whose sides are multiples of 256), in float64 numpy: the
same steps as the tensor-core path takes them, against the oracle's unfolded cosine / sine statement of the field.

  - C[p][n-1-u] = (-1)^p C[p][u] and S[p][n-1-u] = -(-1)^p S[p][u];
  - forward transforms: even frequencies from the folded sum a(u) + a(n-1-u), odd ones from the folded difference,
    over u < n/2, out in the folded frequency order (even frequencies first);
  - the first transform's output folded about the middle of the other axis feeds the second the same way;
  - inverse transforms over a depth in the folded order: E over its first half, O over its second, row m = E + O,
    mirror row n-1-m = E - O for a cosine operand and O - E for a sine one;
  - the row and column weights and the transposed matrices' frequency columns permuted to the folded order.

The GPU tests (test_field_matches_fp64) check the kernels themselves on folded and unfolded grids."""
import numpy as np

from oracle import gp_oracle as O


def _folded(n):
    """Frequency of each position of the folded order."""
    return np.array([2 * c if c < n // 2 else 2 * (c - n // 2) + 1 for c in range(n)])


def _cs(n):
    p = np.arange(n)[:, None]
    u = np.arange(n)[None, :]
    t = np.pi * p * (2 * u + 1) / (2 * n)
    return np.cos(t), np.sin(t)


def _field_folded(a, bin_np):
    nbx, nby = a.shape
    hx, hy = nbx // 2, nby // 2
    cx, sx = _cs(nbx)
    cy, sy = _cs(nby)
    fx, fy = _folded(nbx), _folded(nby)
    wx, wy = O.dct_weights(nbx, nby, bin_np)
    # step 1: the density folded about the middle of y; even / odd y frequencies, rows of Tt in the folded order
    s = a[:, :hy] + a[:, ::-1][:, :hy]
    d = a[:, :hy] - a[:, ::-1][:, :hy]
    tt = np.vstack([cy[0::2, :hy] @ s.T, cy[1::2, :hy] @ d.T])             # [q'][x]
    # its epilogue: Tt folded about the middle of x (sums and differences of the mirrored columns)
    ts = tt[:, :hx] + tt[:, ::-1][:, :hx]
    td = tt[:, :hx] - tt[:, ::-1][:, :hx]
    # step 2: even / odd x frequencies; K in the folded order on both axes, weights permuted alike
    k = np.vstack([cx[0::2, :hx] @ ts.T, cx[1::2, :hx] @ td.T])             # [p'][q']
    kx, ky = k * wx[fx][:, fy], k * wy[fx][:, fy]

    def inverse(at, b, sign):
        """rows m < n/2 of at @ b.T over a folded depth, and their mirrors (sign +1: cosine, -1: sine)."""
        n, h = at.shape[1], at.shape[0] // 2
        e = at[:h, : n // 2] @ b[:, : n // 2].T
        o = at[:h, n // 2:] @ b[:, n // 2:].T
        return np.vstack([e + o, (sign * (e - o))[::-1]])

    # step 3: Pt = CyT' Kx^T (cosine), Qt = SyT' Ky^T (sine); CyT', SyT': frequency columns in the folded order
    pt = inverse(cy.T[:, fy], kx, 1)                                          # [y][p']
    qt = inverse(sy.T[:, fy], ky, -1)
    # step 4: Ex = SxT' Pt^T (sine), Ey = CxT' Qt^T (cosine)
    return inverse(sx.T[:, fx], pt, -1), inverse(cx.T[:, fx], qt, 1)


def test_folded_field_equals_the_unfolded_one():
    rng = np.random.default_rng(3)
    for shape in ((16, 16), (16, 32), (32, 8)):
        a = rng.random(shape) * 0.3 + 0.6
        a[shape[0] // 3, shape[1] // 2] += 40.0
        bin_np = np.array([7.3, 6.1])
        ex, ey = _field_folded(a, bin_np)
        rx, ry = O.field_dct(a, bin_np)
        scale = max(np.abs(rx).max(), np.abs(ry).max())
        assert np.abs(ex - rx).max() <= 1e-12 * scale
        assert np.abs(ey - ry).max() <= 1e-12 * scale


def test_mirror_signs_of_the_cosine_and_sine_matrices():
    n = 12
    c, s = _cs(n)
    sign = (-1.0) ** np.arange(n)[:, None]
    assert np.allclose(c[:, ::-1], sign * c)
    assert np.allclose(s[:, ::-1], -sign * s)
