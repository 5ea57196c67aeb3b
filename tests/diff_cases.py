"""Small cases for the differentiable-render tests (test-only).

`visibility` is a brute-force numpy rasteriser of the continuous model (a
pixel belongs to the nearest front-facing triangle whose perspective-correct
barycentrics at the pixel are all non-negative); it stands in for the exact
rasteriser's visibility in CPU-only tests of the FP64 adjoint."""
import numpy as np

from softlight_gb300 import scenes as S
from oracle import diffrender as D


def visibility(pos, tri, mvp, width, height):
    clip = D.clip_positions(pos, mvp)
    h = clip[tri][:, :, [0, 1, 3]]                 # T x 3 x 3
    z = clip[tri][:, :, 2]
    best = np.full(width * height, np.inf)
    vis = np.zeros(width * height, np.uint32)
    # front-facing: counter-clockwise in NDC
    ndc = h[:, :, :2] / h[:, :, 2:3]
    area = ((ndc[:, 1, 0] - ndc[:, 0, 0]) * (ndc[:, 2, 1] - ndc[:, 0, 1])
            - (ndc[:, 2, 0] - ndc[:, 0, 0]) * (ndc[:, 1, 1] - ndc[:, 0, 1]))
    sx = (ndc[:, :, 0] + 1.0) * 0.5 * width
    sy = (ndc[:, :, 1] + 1.0) * 0.5 * height
    for t in np.nonzero((area > 0) & (h[:, :, 2] > 0).all(1))[0]:
        x0, x1 = max(int(np.floor(sx[t].min())) - 1, 0), min(int(np.ceil(sx[t].max())) + 2, width)
        y0, y1 = max(int(np.floor(sy[t].min())) - 1, 0), min(int(np.ceil(sy[t].max())) + 2, height)
        if x0 >= x1 or y0 >= y1:
            continue
        ys, xs = np.mgrid[y0:y1, x0:x1]
        flat = (ys * width + xs).reshape(-1)
        nx = (2.0 * xs / width - 1.0).reshape(-1)
        ny = (2.0 * ys / height - 1.0).reshape(-1)
        hp_x = h[t, :, 0][None, :] - h[t, :, 2][None, :] * nx[:, None]
        hp_y = h[t, :, 1][None, :] - h[t, :, 2][None, :] * ny[:, None]
        a = [1, 2, 0]
        b = [2, 0, 1]
        e = hp_x[:, a] * hp_y[:, b] - hp_y[:, a] * hp_x[:, b]
        s = e.sum(1)
        lam = e / np.where(s == 0, 1.0, s)[:, None]
        inside = (s != 0) & (lam >= 0).all(1)
        with np.errstate(divide="ignore", invalid="ignore"):
            depth = (lam * z[t][None, :]).sum(1) / (lam * h[t, :, 2][None, :]).sum(1)
        win = inside & (depth < best[flat])
        best[flat[win]] = depth[win]
        vis[flat[win]] = t + 1
    return vis.reshape(height, width)


def small_case(lon=16, lat=8, width=64, height=64, tex_size=16, seed=21):
    pos, uv, idx = S.displaced_sphere(lon, lat, seed)
    uv = S.c5_uv(uv)
    rng = np.random.default_rng(seed)
    col = np.concatenate([rng.uniform(0.3, 1.0, (pos.shape[0], 3)), np.ones((pos.shape[0], 1))], 1)
    tex = S.value_noise(tex_size, tex_size, seed=seed + 1, octaves=2)
    mvp = S.perspective(60.0, width / height, 0.1, 100.0) @ S.look_at((0, 0, 2.5), (0, 0, 0), (0, 1, 0))
    tri = idx.reshape(-1, 3).astype(np.int64)
    vis = visibility(pos.astype(np.float64), tri, mvp, width, height)
    prng = np.random.default_rng(seed + 2)
    target = D.Model(pos + prng.normal(0, 0.01, pos.shape), col + prng.normal(0, 0.05, col.shape), uv, tri,
                     tex + prng.normal(0, 0.05, tex.shape), mvp, vis).image()
    return dict(pos=pos.astype(np.float64), col=col, uv=uv.astype(np.float64), tri=tri, tex=tex, mvp=mvp,
                vis=vis, target=target)
