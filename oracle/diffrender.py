"""FP64 CPU restatement of the differentiable shading model and its adjoint.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline as the checker of the GPU adjoint, never by the
product path.

SoftLight has no adjoint; what is differentiated here is its forward shading
of one opaque draw of the vertex-colour x float-texture program, over the
coverage the exact rasteriser produced (the per-pixel visible triangle):

  * sample point: pixel (x, y) at integer screen coordinates, as the
    reference's scan-line loop evaluates it (softlight/src/SL_TriRasterizer.cpp:
    807-923); in NDC n = (2x/W - 1, 2y/H - 1) for the full-framebuffer
    viewport (softlight/src/SL_ViewportState.cpp:17-110);
  * perspective-correct barycentrics of the triangle's clip-space vertices
    h_k = (x, y, w) at n: e_k = det(h_{k+1}, h_{k+2}, n), l_k = e_k / sum(e),
    the closed form of the reference's screen barycentrics times 1/w, then
    renormalised (softlight/src/SL_FragmentProcessor.cpp:463-529), taken at
    the unsnapped vertex positions so that positions have interior
    derivatives (the reference floors screen positions,
    softlight/include/softlight/SL_PostVertexTransform.hpp:509-524);
  * varyings colour = sum l_k C_k, uv = sum l_k UV_k
    (interpolate_tri_varyings, SL_FragmentProcessor.cpp:308-330);
  * bilinear REPEAT sampling of an RGBA float texture with the reference's
    texel addressing: x = wrap(u) W, x0 = trunc(x), x1 = min(x0 + 1, W),
    linear index x + W y into the texel array followed by zero padding
    (softlight/include/softlight/SL_Sampler.hpp:97-218);
  * output = colour * texel (componentwise);
  * domain: a visible pixel is modelled when every barycentric is >= -1
    (within one triangle height of the unsnapped triangle; snapping lets
    slivers own pixels far outside their unsnapped shape, where the
    extrapolation is ill-conditioned) and its triangle is not a sliver in the
    h' frame: |sum e_k| >= 0.02 x the sum of its squared edge lengths
    (barycentrics vary as 1/area, so near-degenerate and edge-on triangles
    have unbounded sensitivity). Other pixels keep the framebuffer's colour
    and carry no gradient.

The adjoint takes dL/d(output) per pixel and returns dL/d positions (V x 3),
colours (V x 4), uvs (V x 2) and texels (H x W x 4). Texel indices that fall
in the padding are constants and receive no gradient.
"""
import numpy as np


def clip_positions(pos, mvp):
    """Clip-space (x, y, z, w) of object positions (V x 3); mvp is the 4x4
    row-major matrix M with clip = M @ (p, 1)."""
    p = np.concatenate([pos.astype(np.float64), np.ones((pos.shape[0], 1))], 1)
    return p @ np.asarray(mvp, np.float64).T


MIN_BARYCENTRIC = -1.0
MIN_SHAPE = 0.02   # |2 x area| / (sum of squared edge lengths); 0.29 for an equilateral triangle


def wrap_repeat(t):
    return (t < 0).astype(np.float64) + np.fmod(t, 1.0)


class Model:
    """Per-pixel intermediates of the forward model for one visibility map."""

    def __init__(self, pos, col, uv, tri, tex, mvp, vis, frozen=None):
        self.pos = np.asarray(pos, np.float64)
        self.col = np.asarray(col, np.float64)
        self.uv = np.asarray(uv, np.float64)
        self.tri = np.asarray(tri, np.int64).reshape(-1, 3)
        self.tex = np.asarray(tex, np.float64)
        self.mvp = np.asarray(mvp, np.float64)
        self.vis = np.asarray(vis, np.uint32)
        self.H, self.W = self.vis.shape
        self.TH, self.TW = self.tex.shape[:2]
        self._forward(frozen)

    def _forward(self, frozen):
        """frozen: a Model whose discrete choices are kept -- the covered
        pixels, the repeat offset of each uv and the bilinear texel cell --
        so that finite differences see the smooth function the adjoint
        differentiates."""
        H, W = self.H, self.W
        ids = self.vis.reshape(-1).astype(np.int64) - 1
        pix = np.nonzero((ids >= 0) & (ids < self.tri.shape[0]))[0]
        t = ids[pix]
        self.pix, self.t = pix, t
        ys, xs = np.divmod(pix, W)
        nx = 2.0 * xs / W - 1.0
        ny = 2.0 * ys / H - 1.0
        clip = clip_positions(self.pos, self.mvp)
        v = self.tri[t]                              # P x 3 vertex ids
        h = clip[v][:, :, [0, 1, 3]]                 # P x 3 x (x, y, w)
        # h' = h - w n (x, y): det(a, b, n) = cross2(a', b')
        hp = np.stack([h[:, :, 0] - h[:, :, 2] * nx[:, None], h[:, :, 1] - h[:, :, 2] * ny[:, None]], -1)
        a, b = np.roll(hp, -1, axis=1), np.roll(hp, -2, axis=1)   # h'_{k+1}, h'_{k+2}
        e = a[:, :, 0] * b[:, :, 1] - a[:, :, 1] * b[:, :, 0]
        S = e.sum(1)
        if frozen is None:
            # squared edge lengths of the triangle in the h' frame
            e2 = sum(((np.roll(hp, -1, axis=1) - hp) ** 2).sum(2).T)
            with np.errstate(divide="ignore", invalid="ignore"):
                ok = ((S != 0.0) & ((e / np.where(S == 0.0, 1.0, S)[:, None]).min(1) >= MIN_BARYCENTRIC)
                      & (np.abs(S) >= MIN_SHAPE * e2))
        else:
            ok = np.isin(pix, frozen.pix)
        self.pix, self.t, v, h, hp, a, b, e, S = pix[ok], t[ok], v[ok], h[ok], hp[ok], a[ok], b[ok], e[ok], S[ok]
        nx, ny = nx[ok], ny[ok]
        lam = e / S[:, None]
        C = self.col[v]                              # P x 3 x 4
        U = self.uv[v]                               # P x 3 x 2
        colour = (lam[:, :, None] * C).sum(1)
        uvs = (lam[:, :, None] * U).sum(1)

        TW, TH = self.TW, self.TH
        if frozen is None:
            self.wrap_u = wrap_repeat(uvs[:, 0]) - uvs[:, 0]
            self.wrap_v = wrap_repeat(uvs[:, 1]) - uvs[:, 1]
            xf = wrap_repeat(uvs[:, 0]) * TW
            yf = wrap_repeat(uvs[:, 1]) * TH
            xi0 = np.trunc(xf).astype(np.int64) & 0xFFFF
            yi0 = np.trunc(yf).astype(np.int64) & 0xFFFF
        else:
            self.wrap_u, self.wrap_v = frozen.wrap_u, frozen.wrap_v
            xf = (uvs[:, 0] + self.wrap_u) * TW
            yf = (uvs[:, 1] + self.wrap_v) * TH
            xi0, yi0 = frozen.xi0, frozen.yi0
        self.xi0, self.yi0 = xi0, yi0
        xi1 = np.minimum((xi0 + 1) & 0xFFFF, TW)
        yi1 = np.minimum((yi0 + 1) & 0xFFFF, TH)
        dx, dy = xf - xi0, yf - yi0
        idx = np.stack([xi0 + TW * yi0, xi0 + TW * yi1, xi1 + TW * yi0, xi1 + TW * yi1], 1)   # 00, 01, 10, 11
        wts = np.stack([(1 - dx) * (1 - dy), (1 - dx) * dy, dx * (1 - dy), dx * dy], 1)
        flat = np.concatenate([self.tex.reshape(-1, 4), np.zeros((TW + 64, 4))], 0)
        T = flat[idx]                                # P x 4 x 4
        texel = (wts[:, :, None] * T).sum(1)

        self.v, self.h, self.hp, self.a, self.b, self.e, self.S = v, h, hp, a, b, e, S
        self.nx, self.ny, self.lam, self.C, self.U = nx, ny, lam, C, U
        self.colour, self.uvs, self.texel = colour, uvs, texel
        self.idx, self.wts, self.T, self.dx, self.dy = idx, wts, T, dx, dy
        self.out = colour * texel

    def image(self, fill=None):
        """Model image; pixels outside the model take `fill` (H x W x 4,
        the framebuffer's colour) or 0."""
        img = np.zeros((self.H * self.W, 4)) if fill is None else np.array(fill, np.float64).reshape(-1, 4)
        img[self.pix] = self.out
        return img.reshape(self.H, self.W, 4)

    def adjoint(self, d_image):
        """Gradients for dL/d(image) (H x W x 4): (dpos, dcol, duv, dtex)."""
        g = np.asarray(d_image, np.float64).reshape(-1, 4)[self.pix]
        V = self.pos.shape[0]
        gc = g * self.texel                          # dL/d colour varying
        gt = g * self.colour                         # dL/d texel sample
        TW, TH = self.TW, self.TH
        T = self.T
        dS_ddx = -(1 - self.dy)[:, None] * T[:, 0] - self.dy[:, None] * T[:, 1] + (1 - self.dy)[:, None] * T[:, 2] + self.dy[:, None] * T[:, 3]
        dS_ddy = -(1 - self.dx)[:, None] * T[:, 0] + (1 - self.dx)[:, None] * T[:, 1] - self.dx[:, None] * T[:, 2] + self.dx[:, None] * T[:, 3]
        duv = np.stack([(gt * dS_ddx).sum(1) * TW, (gt * dS_ddy).sum(1) * TH], 1)

        dcol = np.zeros((V, 4))
        duvv = np.zeros((V, 2))
        np.add.at(dcol, self.v.reshape(-1), (self.lam[:, :, None] * gc[:, None, :]).reshape(-1, 4))
        np.add.at(duvv, self.v.reshape(-1), (self.lam[:, :, None] * duv[:, None, :]).reshape(-1, 2))

        dtex = np.zeros((TW * TH + TW + 64, 4))
        np.add.at(dtex, self.idx.reshape(-1), (self.wts[:, :, None] * gt[:, None, :]).reshape(-1, 4))
        dtex = dtex[:TW * TH].reshape(TH, TW, 4)

        dlam = (gc[:, None, :] * self.C).sum(2) + (duv[:, None, :] * self.U).sum(2)      # P x 3
        de = (dlam - (self.lam * dlam).sum(1, keepdims=True)) / self.S[:, None]
        a, b = self.a, self.b
        # e_k = a_k.x b_k.y - a_k.y b_k.x with a_k = h'_{k+1}, b_k = h'_{k+2}
        da = np.stack([b[:, :, 1], -b[:, :, 0]], -1) * de[:, :, None]
        db = np.stack([-a[:, :, 1], a[:, :, 0]], -1) * de[:, :, None]
        dhp = np.roll(da, 1, axis=1) + np.roll(db, 2, axis=1)                              # P x 3 x 2
        dw = -(dhp[:, :, 0] * self.nx[:, None] + dhp[:, :, 1] * self.ny[:, None])
        dclip = np.stack([dhp[:, :, 0], dhp[:, :, 1], np.zeros_like(dw), dw], -1)           # P x 3 x 4
        dp = dclip.reshape(-1, 4) @ self.mvp[:, :3]                                          # d pos = M[:, :3]^T dclip
        dpos = np.zeros((V, 3))
        np.add.at(dpos, self.v.reshape(-1), dp)
        return dpos, dcol, duvv, dtex


def l2_loss(img, target, covered):
    """Sum of squared differences over the covered pixels."""
    d = (img - target)[covered]
    return float((d * d).sum())


def loss_and_grad(pos, col, uv, tri, tex, mvp, vis, target):
    m = Model(pos, col, uv, tri, tex, mvp, vis)
    covered = np.zeros(m.H * m.W, bool)
    covered[m.pix] = True
    covered = covered.reshape(m.H, m.W)
    img = m.image()
    d_img = np.where(covered[..., None], 2.0 * (img - target), 0.0)
    return l2_loss(img, target, covered), m.adjoint(d_img)


def loss_only(pos, col, uv, tri, tex, mvp, vis, target, frozen=None):
    m = Model(pos, col, uv, tri, tex, mvp, vis, frozen)
    covered = np.zeros(m.H * m.W, bool)
    covered[m.pix] = True
    return l2_loss(m.image(), target, covered.reshape(m.H, m.W))
