"""The column pass's candidate columns (columns.cu, columnRasterKernel and launchSignColumns): for a
triangle, the columns whose FP32 centre (x, y) lies in the triangle's closed (x, y) bounds must all be
candidates, however the grid is placed, scaled or turned about z and however far from the origin.  This
restates the candidate arithmetic in numpy FP32 (the widening by twice the centres' rounding, the FP32
map to index space with its 1e-6 relative margin) and checks it on random triangles against the
centres computed the way the grid computes them (left-to-right dots, FP32)."""
import math

import numpy as np

f32 = np.float32


def centres(xf, ix, iy):
    a0, a1, a3, a4, b0, b1 = (f32(xf[k]) for k in (0, 1, 3, 4, 9, 10))
    fx, fy = ix.astype(f32), iy.astype(f32)
    # (a0 x + a1 y) + a2 z with a2 = 0, then + b: the grid's left-to-right dot in FP32
    X = ((a0 * fx + a1 * fy) + f32(0)) + b0
    Y = ((a3 * fx + a4 * fy) + f32(0)) + b1
    return X.astype(f32), Y.astype(f32)


def candidates(xf, nx, ny, tri):
    a0, a1, a3, a4 = (float(xf[k]) for k in (0, 1, 3, 4))
    det = a0 * a4 - a1 * a3
    inv = [f32(a4 / det), f32(-a1 / det), f32(-a3 / det), f32(a0 / det)]
    org = [f32(xf[9]), f32(xf[10])]

    def margin(m):
        m = m if m > 0 else 1e-30
        return f32(4.0 * math.ldexp(1.0, math.frexp(m)[1] - 1 - 23))
    ex = margin(abs(a0) * (nx - 1) + abs(a1) * (ny - 1) + abs(float(xf[9])))
    ey = margin(abs(a3) * (nx - 1) + abs(a4) * (ny - 1) + abs(float(xf[10])))
    x0 = f32(f32(tri[:, 0].min() - ex) - org[0])
    x1 = f32(f32(tri[:, 0].max() - org[0]) + ex)
    y0 = f32(f32(tri[:, 1].min() - ey) - org[1])
    y1 = f32(f32(tri[:, 1].max() - org[1]) + ey)
    fx0 = fy0 = np.inf
    fx1 = fy1 = -np.inf
    for c in range(4):
        X = x1 if c & 1 else x0
        Y = y1 if c & 2 else y0
        tx = abs(f32(inv[0] * X)) + abs(f32(inv[1] * Y))
        ty = abs(f32(inv[2] * X)) + abs(f32(inv[3] * Y))
        fx = f32(float(inv[0]) * float(X) + float(f32(inv[1] * Y)))  # the kernel's fmaf
        fy = f32(float(inv[2]) * float(X) + float(f32(inv[3] * Y)))
        fx0, fx1 = min(fx0, f32(fx - f32(1e-6) * tx)), max(fx1, f32(fx + f32(1e-6) * tx))
        fy0, fy1 = min(fy0, f32(fy - f32(1e-6) * ty)), max(fy1, f32(fy + f32(1e-6) * ty))
    return (max(0, math.ceil(fx0)), min(nx - 1, math.floor(fx1)), max(0, math.ceil(fy0)), min(ny - 1, math.floor(fy1)))


def test_candidate_columns_cover_the_triangle_bounds():
    rng = np.random.default_rng(0)
    checked = 0
    for trial in range(300):
        n = int(rng.integers(8, 64))
        pitch = float(10.0 ** rng.uniform(-4, 1))
        angle = rng.uniform(0, 2 * math.pi) if trial % 2 else 0.0
        origin = rng.uniform(-1, 1, 2) * 10.0 ** rng.uniform(0, 4)
        c, s = math.cos(angle), math.sin(angle)
        sx, sy = pitch, pitch * rng.uniform(0.5, 2.0)
        xf = np.zeros(12, np.float32)
        xf[0], xf[1], xf[3], xf[4] = c * sx, -s * sy, s * sx, c * sy
        xf[8] = pitch
        xf[9], xf[10] = origin
        ix, iy = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        X, Y = centres(xf, ix.ravel(), iy.ravel())
        for _ in range(20):
            # a triangle inside the grid's footprint, some with a vertex exactly on a column centre
            k = rng.integers(0, n * n, 3)
            tri = np.stack([X[k] + (rng.uniform(-1, 1, 3) * pitch * rng.uniform(0, 3)).astype(f32) * (rng.random(3) < 0.7),
                            Y[k] + (rng.uniform(-1, 1, 3) * pitch * rng.uniform(0, 3)).astype(f32) * (rng.random(3) < 0.7)],
                           1).astype(f32)
            inside = (X >= tri[:, 0].min()) & (X <= tri[:, 0].max()) & (Y >= tri[:, 1].min()) & (Y <= tri[:, 1].max())
            cx0, cx1, cy0, cy1 = candidates(xf, n, n, tri)
            ii, jj = ix.ravel()[inside], iy.ravel()[inside]
            assert np.all((ii >= cx0) & (ii <= cx1) & (jj >= cy0) & (jj <= cy1)), (trial, xf, tri)
            checked += int(inside.sum())
    assert checked > 1000
