"""torch.autograd.Function over the differentiable-render C ABI (test harness).

forward(pos, col, tex) uploads the parameters into the scene's vertex buffer
and texture, renders the draw with the exact rasteriser into a framebuffer
with a visibility map, and returns the model image (slg_diff_shade);
backward(dL/d image) runs slg_draw_adjoint, which recomputes the forward per
pixel, and returns dL/d positions, colours and texels. torch provides device
memory and the autograd plumbing only. backward uses the visibility map and
parameters of the most recent forward on the same scene."""
import torch


class DiffRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, col, tex, scene):
        scene.set_params(pos.detach().cpu().numpy(), col.detach().cpu().numpy(), tex.detach().cpu().numpy())
        c = scene.ctx
        c.clear_framebuffer(scene.fbo, 0, scene.clear_color, scene.clear_depth)
        c.draw(scene.mesh, scene.shader, scene.fbo)
        img = torch.empty(scene.height, scene.width, 4, device=pos.device, dtype=torch.float32)
        torch.cuda.synchronize()
        c.diff_shade(scene.mesh, scene.shader, scene.fbo, img.data_ptr(), img.numel())
        c.finish()
        ctx.scene = scene
        return img

    @staticmethod
    def backward(ctx, grad):
        s = ctx.scene
        g = grad.contiguous().float()
        nv = s.pos.shape[0]
        dvert = torch.zeros(nv * 9, device=g.device, dtype=torch.float32)
        dtex = torch.zeros(s.tex.size, device=g.device, dtype=torch.float32)
        torch.cuda.synchronize()
        s.ctx.draw_adjoint(s.mesh, s.shader, s.fbo, g.data_ptr(), g.numel(), dvert.data_ptr(), dvert.numel(),
                           dtex.data_ptr(), dtex.numel())
        s.ctx.finish()
        dv = dvert.view(nv, 9)
        return dv[:, :3].contiguous(), dv[:, 3:7].contiguous(), dtex.view(*s.tex.shape), None


def render(scene, pos, col, tex):
    return DiffRender.apply(pos, col, tex, scene)
