"""GPU tests of the differentiable render (slg_fbo_enable_visibility,
slg_diff_shade, slg_draw_adjoint) against the FP64 CPU model and adjoint in
oracle/diffrender.py, evaluated on the visibility map the GPU's exact
rasteriser recorded, and against central finite differences.

Tolerances, all norm-wise relative errors:
  * model image, GPU FP32 vs FP64: 1e-5;
  * gradients (positions, colours, uvs, texels), GPU FP32 adjoint vs FP64
    adjoint: 1e-4;
  * GPU gradients vs central differences (h = 1e-3) of the FP64 loss with
    coverage, uv repeat offsets and texel cells frozen, on 64 sampled
    parameters: colours and texels 1e-4 (the loss is quadratic in them, so
    the differences are exact). Positions enter through barycentrics that
    vary as 1/area, and triangles near the silhouette and the poles project
    to a few pixels, where a 1e-3 step changes their screen area by tens of
    percent: h = 1e-3 carries up to ~4% O(h^2) truncation error there, so
    its bound is 0.1, the Richardson combination of h and h/2 is held to
    1e-2, and FP64 central differences at h = 1e-5 (truncation ~1e-6,
    rounding ~1e-10) to 1e-4."""
import numpy as np
import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S
from oracle import diffrender as D

torch = pytest.importorskip("torch")
import diff_harness  # noqa: E402

pytestmark = pytest.mark.gpu

SMALL = dict(width=96, height=80, tex_size=16, lon=16, lat=8)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def mvp32(s):
    return S.col_major(s.mvp).astype(np.float64).reshape(4, 4).T


def frame(s):
    c = s.ctx
    c.clear_framebuffer(s.fbo, 0, s.clear_color, s.clear_depth)
    c.draw(s.mesh, s.shader, s.fbo)
    img = torch.empty(s.height, s.width, 4, device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    c.diff_shade(s.mesh, s.shader, s.fbo, img.data_ptr(), img.numel())
    c.finish()
    return img, c.fbo_read_visibility(s.fbo, (s.height, s.width))


def target_image(s):
    keep = (s.pos.copy(), s.col.copy(), s.tex.copy())
    s.set_params(*S.c5_perturbed(s))
    img, _ = frame(s)
    s.set_params(*keep)
    return img


def gpu_adjoint(s, d_img):
    nv = s.pos.shape[0]
    dvert = torch.zeros(nv * 9, device="cuda", dtype=torch.float32)
    dtex = torch.zeros(s.tex.size, device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    s.ctx.draw_adjoint(s.mesh, s.shader, s.fbo, d_img.data_ptr(), d_img.numel(), dvert.data_ptr(), dvert.numel(),
                       dtex.data_ptr(), dtex.numel())
    s.ctx.finish()
    dv = dvert.view(nv, 9).cpu().numpy()
    return dv[:, :3], dv[:, 3:7], dv[:, 7:9], dtex.view(*s.tex.shape).cpu().numpy()


def oracle_model(s, vis, frozen=None):
    return D.Model(s.pos, s.col, s.uv, s.tri, s.tex, mvp32(s), vis, frozen)


@pytest.fixture(scope="module")
def c5(gpu_lib):
    ctx = gpu_lib.Context()
    s = S.build_c5(ctx)
    target = target_image(s)
    img, vis = frame(s)
    yield s, img, vis, target
    ctx.close()


def test_visibility_is_the_exact_coverage(c5):
    s, img, vis, _ = c5
    depth = s.read_depth()
    assert ((vis > 0) == (depth < s.clear_depth)).all()
    assert vis.max() <= s.num_triangles
    assert (vis > 0).sum() > 50000


def test_model_image_matches_fp64(c5):
    s, img, vis, _ = c5
    m = oracle_model(s, vis)
    exact = s.read_color()
    want = m.image(fill=exact)
    got = img.cpu().numpy()
    assert rel(got, want) <= 1e-5
    assert np.abs(got - want).max() <= 1e-4
    # the model departs from the exact draw's colours only by the sub-pixel
    # snapping of vertex positions
    assert np.abs(exact - want).mean() < 0.05
    assert len(m.pix) > 0.99 * (vis > 0).sum()


def test_adjoint_matches_fp64(c5):
    s, img, vis, target = c5
    d_img = (2.0 * (img - target)).contiguous()
    got = gpu_adjoint(s, d_img)
    want = oracle_model(s, vis).adjoint(d_img.cpu().numpy().astype(np.float64))
    for name, g, w in zip(("pos", "col", "uv", "tex"), got, want):
        assert np.linalg.norm(w) > 0, name
        assert rel(g, w) <= 1e-4, f"{name}: GPU vs FP64 adjoint relative error {rel(g, w):.3e}"


def test_adjoint_accumulates(c5):
    s, img, vis, target = c5
    d_img = (2.0 * (img - target)).contiguous()
    nv = s.pos.shape[0]
    dvert = torch.zeros(nv * 9, device="cuda")
    dtex = torch.zeros(s.tex.size, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        s.ctx.draw_adjoint(s.mesh, s.shader, s.fbo, d_img.data_ptr(), d_img.numel(), dvert.data_ptr(), dvert.numel(),
                           dtex.data_ptr(), dtex.numel())
    s.ctx.finish()
    once = gpu_adjoint(s, d_img)
    assert rel(dvert.view(nv, 9)[:, 3:7].cpu().numpy(), 2.0 * once[1]) <= 1e-5
    assert rel(dtex.view(*s.tex.shape).cpu().numpy(), 2.0 * once[3]) <= 1e-5


def fd(s, vis, target, base, name, index, h):
    def loss(delta):
        p = {"pos": s.pos.astype(np.float64), "col": s.col.astype(np.float64), "tex": s.tex.astype(np.float64)}
        p[name] = p[name].copy()
        p[name].reshape(-1)[index] += delta
        return D.loss_only(p["pos"], p["col"], s.uv, s.tri, p["tex"], mvp32(s), vis, target, frozen=base)
    return (loss(h) - loss(-h)) / (2.0 * h)


def test_autograd_harness_against_fp64_and_differences(c5):
    s, _, _, target = c5
    pos = torch.tensor(s.pos, device="cuda", requires_grad=True)
    col = torch.tensor(s.col, device="cuda", requires_grad=True)
    tex = torch.tensor(s.tex, device="cuda", requires_grad=True)
    img = diff_harness.render(s, pos, col, tex)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    vis = s.ctx.fbo_read_visibility(s.fbo, (s.height, s.width))
    tgt = target.cpu().numpy().astype(np.float64)
    base = oracle_model(s, vis)
    # uncovered pixels hold 0 in the model image: their residual is constant in the parameters
    _, want = D.loss_and_grad(s.pos, s.col, s.uv, s.tri, s.tex, mvp32(s), vis, tgt)
    grads = {"pos": pos.grad.cpu().numpy(), "col": col.grad.cpu().numpy(), "tex": tex.grad.cpu().numpy()}
    for name, w in (("pos", want[0]), ("col", want[1]), ("tex", want[3])):
        assert rel(grads[name], w) <= 1e-4, f"{name}: autograd vs FP64 adjoint {rel(grads[name], w):.3e}"

    # 64 sampled parameters: 22 colour, 21 texel and 21 position components
    rng = np.random.default_rng(7)
    for name, tol, count in (("col", 1e-4, 22), ("tex", 1e-4, 21), ("pos", 0.1, 21)):
        g = grads[name].reshape(-1)
        cand = np.nonzero(np.abs(g) > 1e-2 * np.abs(g).max())[0]
        idx = rng.choice(cand, size=count, replace=False)
        num = np.array([fd(s, vis, tgt, base, name, i, 1e-3) for i in idx])
        err = rel(g[idx], num)
        assert err <= tol, f"{name}: GPU gradient vs central differences {err:.3e}"
        if name == "pos":
            num2 = np.array([fd(s, vis, tgt, base, name, i, 5e-4) for i in idx])
            err = rel(g[idx], (4.0 * num2 - num) / 3.0)
            assert err <= 1e-2, f"pos: GPU gradient vs Richardson differences {err:.3e}"
            fine = np.array([fd(s, vis, tgt, base, name, i, 1e-5) for i in idx])
            err = rel(g[idx], fine)
            assert err <= 1e-4, f"pos: GPU gradient vs central differences at h=1e-5 {err:.3e}"


@pytest.mark.parametrize("index_dtype", [np.uint8, np.uint16, np.uint32, None])
def test_index_types_and_small_frames(gpu_lib, index_dtype):
    ctx = gpu_lib.Context()
    try:
        s = S.build_c5(ctx, index_dtype=index_dtype, **SMALL)
        target = target_image(s)
        img, vis = frame(s)
        assert (vis > 0).sum() > 500
        d_img = (2.0 * (img - target)).contiguous()
        got = gpu_adjoint(s, d_img)
        want = oracle_model(s, vis).adjoint(d_img.cpu().numpy().astype(np.float64))
        for name, g, w in zip(("pos", "col", "uv", "tex"), got, want):
            assert rel(g, w) <= 1e-4, f"{name} ({index_dtype}): {rel(g, w):.3e}"
    finally:
        ctx.close()


def test_rejections(gpu_lib):
    ctx = gpu_lib.Context()
    try:
        s = S.build_c5(ctx, **SMALL)
        img, _ = frame(s)
        nv = s.pos.shape[0]
        dvert = torch.zeros(nv * 9, device="cuda")
        dtex = torch.zeros(s.tex.size, device="cuda")
        small = torch.zeros(nv * 9 - 1, device="cuda")
        host = np.zeros(img.numel(), np.float32)
        args = (img.data_ptr(), img.numel(), dvert.data_ptr(), dvert.numel(), dtex.data_ptr(), dtex.numel())
        with pytest.raises(A.SLError, match="dVertices"):
            ctx.draw_adjoint(s.mesh, s.shader, s.fbo, img.data_ptr(), img.numel(), small.data_ptr(), small.numel(),
                             dtex.data_ptr(), dtex.numel())
        with pytest.raises(A.SLError, match="dImage"):
            ctx.draw_adjoint(s.mesh, s.shader, s.fbo, host.ctypes.data, host.size, *args[2:])
        with pytest.raises(A.SLError, match="dTexels"):
            ctx.draw_adjoint(s.mesh, s.shader, s.fbo, *args[:4], dtex.data_ptr(), dtex.numel() - 4)
        # a framebuffer with a visibility map takes opaque draws only
        blend_sh = s.add_shader(A.PROGRAM_VCOLOR_TEXF, 2, S.vcolor_uniforms(s.mvp, s.tex_id), blend=A.BLEND_ALPHA)
        with pytest.raises(A.SLError, match="opaque"):
            ctx.draw(s.mesh, blend_sh, s.fbo)
        # another program is outside the model
        other = S.build_c1(ctx, width=64, height=48)
        ctx.fbo_enable_visibility(other.fbo)
        mesh, _, sh = other.draws[0]
        with pytest.raises(A.SLError, match="VCOLOR_TEXF"):
            ctx.draw_adjoint(mesh, sh, other.fbo, *args)
        # no visibility map
        ctx.fbo_enable_visibility(s.fbo, False)
        with pytest.raises(A.SLError, match="visibility"):
            ctx.draw_adjoint(s.mesh, s.shader, s.fbo, *args)
        ctx.finish()
    finally:
        ctx.close()
