"""GPU tests of the differentiable march: forward images against the renderer
and the CPU oracle (bit for bit), hand-written backward against PyTorch
autograd of the reference marcher and against float64 central finite
differences (h = 1e-4) on a 32^3 volume / 64^2 image sub-case, and a short
transfer-function recovery with Adam."""

import numpy as np
import pytest

import oracle
from oracle import march_torch
from pyvr_gb300 import Camera, Light, RenderConfig, Volume, VolumeRenderer, compute_normal_volume
from pyvr_gb300 import workloads as W
from pyvr_gb300.diff import DiffScene, render_views
from pyvr_gb300.renderer import rgba_lut

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _case(n=32, res=64, views=2, normals=True, seed=3, opacity=0.3):
    data = W.value_noise((n, n, n), seed=seed).astype(np.float32)
    nrm = compute_normal_volume(data) if normals else None
    rng = np.random.default_rng(seed)
    ctf = W.standin_colormap(seed % 12)
    lut0 = rgba_lut(ctf, W.random_opacity(rng, 8, opacity))
    lut1 = rgba_lut(ctf, W.random_opacity(rng, 8, opacity))
    cams = [Camera.from_spherical(np.zeros(3, np.float32), 2 * np.pi * k / views + 0.3, 0.5, 0.0, 3.0)
            for k in range(views)]
    light = Light.directional([1, -1, 0], 0.2, 0.8)
    cfg = RenderConfig.balanced()
    scene = DiffScene(cams, light, cfg, res, res)
    vol = Volume(data=data, normals=nrm, min_bounds=np.full(3, -1.0, np.float32),
                 max_bounds=np.full(3, 1.0, np.float32))
    frames = [W.frame_inputs(vol, c, light, cfg, lut0, res, res) for c in cams]
    return dict(data=data, nrm=nrm, lut0=lut0, lut1=lut1, cams=cams, light=light, cfg=cfg, scene=scene,
                vol=vol, frames=frames, res=res)


def _dev(a, grad=False):
    return torch.tensor(a, device="cuda", requires_grad=grad)


@pytest.mark.parametrize("normals", [True, False])
def test_forward_equals_renderer_and_oracle(normals):
    c = _case(views=3, normals=normals)
    nrm = _dev(c["nrm"]) if normals else None
    img = render_views(_dev(c["data"]), _dev(c["lut0"]), c["scene"], nrm).cpu().numpy()
    for k, (cam, s) in enumerate(zip(c["cams"], c["frames"])):
        _, of, _ = oracle.render(s)
        assert np.array_equal(img[k].view(np.uint32), of.view(np.uint32)), k
        with VolumeRenderer(c["res"], c["res"], config=c["cfg"], light=c["light"]) as r:
            r.load_volume(c["vol"])
            r.set_camera(cam)
            r.set_transfer_functions(*_tfs_for(c))
            _, gf = r.render_float()
        assert np.array_equal(img[k].view(np.uint32), np.asarray(gf).view(np.uint32)), k


def _tfs_for(c):
    """Transfer functions whose table is exactly lut0 (piecewise linear through its entries)."""
    from pyvr_gb300 import ColorTransferFunction, OpacityTransferFunction
    lut = c["lut0"]
    xs = np.linspace(0.0, 1.0, lut.shape[0])
    ctf = ColorTransferFunction([(float(x), tuple(float(v) for v in lut[i, :3])) for i, x in enumerate(xs)])
    otf = OpacityTransferFunction([(float(x), float(lut[i, 3])) for i, x in enumerate(xs)])
    return ctf, otf


def _loss_grads_kernel(c, target, normals, want_vol=True, want_lut=True):
    vol = _dev(c["data"], want_vol)
    lut = _dev(c["lut0"], want_lut)
    nrm = _dev(c["nrm"]) if normals else None
    img = render_views(vol, lut, c["scene"], nrm)
    loss = ((img - target.cuda()) ** 2).mean()
    loss.backward()
    return (loss.item(), vol.grad.cpu().numpy() if want_vol else None,
            lut.grad.cpu().numpy() if want_lut else None)


def _target(c):
    with torch.no_grad():
        nrm = _dev(c["nrm"]) if c["nrm"] is not None else None
        return render_views(_dev(c["data"]), _dev(c["lut1"]), c["scene"], nrm).cpu()


@pytest.mark.parametrize("normals", [True, False])
def test_backward_matches_torch_autograd(normals):
    c = _case(normals=normals)
    target = _target(c)
    loss_k, gv_k, gl_k = _loss_grads_kernel(c, target, normals)
    vol = torch.tensor(c["data"], requires_grad=True)
    lut = torch.tensor(c["lut0"], requires_grad=True)
    nrm = torch.tensor(c["nrm"]) if normals else None
    img, _ = march_torch.render_views(vol, lut, c["frames"], nrm, torch.float32)
    loss = ((img - target) ** 2).mean()
    loss.backward()
    gv_t, gl_t = vol.grad.numpy(), lut.grad.numpy()
    assert abs(loss_k - loss.item()) <= 1e-5 * loss.item()
    for name, gk, gt in (("lut", gl_k, gl_t), ("volume", gv_k, gv_t)):
        assert np.abs(gt).max() > 0, name
        rel = np.linalg.norm(gk - gt) / np.linalg.norm(gt)
        assert rel < 2e-3, (name, rel)
        assert np.abs(gk - gt).max() <= 1e-2 * np.abs(gt).max(), name


def test_backward_matches_fp64_central_differences():
    # 32^3 volume, one 64^2 view, h = 1e-4 in float64.  Opacities low enough
    # that no ray reaches the 0.99 termination: the loss is then a continuous
    # function of the LUT and the voxels (a ray that terminates one sample
    # earlier or later under +-h would add a jump that no gradient describes)
    c = _case(views=1, opacity=0.02)
    target = _target(c)
    assert float(target[..., 3].max()) < 0.98
    _, gv, gl = _loss_grads_kernel(c, target, True)
    nrm = torch.tensor(c["nrm"])
    t64 = target.double()

    def loss(v, l):
        img, _ = march_torch.render_views(v, l, c["frames"], nrm, torch.float64)
        return ((img - t64) ** 2).mean().item()

    v0 = torch.tensor(c["data"], dtype=torch.float64)
    l0 = torch.tensor(c["lut0"], dtype=torch.float64)
    h = 1e-4
    picks = [("lut", np.unravel_index(i, gl.shape)) for i in np.argsort(-np.abs(gl).ravel())[:6]]
    picks += [("vol", np.unravel_index(i, gv.shape)) for i in np.argsort(-np.abs(gv).ravel())[:6]]
    errs = []
    for which, idx in picks:
        vp, vm, lp, lm = v0.clone(), v0.clone(), l0.clone(), l0.clone()
        if which == "lut":
            lp[idx] += h
            lm[idx] -= h
            g = gl[idx]
        else:
            vp[idx] += h
            vm[idx] -= h
            g = gv[idx]
        fd = (loss(vp, lp) - loss(vm, lm)) / (2 * h)
        errs.append((which, idx, fd, float(g)))
        assert abs(fd - g) <= 1e-2 * abs(fd) + 1e-3 * max(np.abs(gl).max(), np.abs(gv).max()), errs[-1]


def test_gradient_selection_and_many_views():
    # 40 views (two launches) equal the views rendered alone; a LUT-only
    # backward leaves the volume without gradient
    c = _case(n=12, res=16, views=40)
    vol, lut, nrm = _dev(c["data"]), _dev(c["lut0"], True), _dev(c["nrm"])
    img = render_views(vol, lut, c["scene"], nrm)
    for k in (0, 33, 39):
        one = DiffScene([c["cams"][k]], c["light"], c["cfg"], 16, 16)
        assert torch.equal(render_views(vol, lut, one, nrm)[0], img[k])
    img.square().mean().backward()
    assert vol.grad is None and lut.grad is not None and lut.grad.abs().sum() > 0


def test_adam_recovers_transfer_function():
    c = _case(views=4)
    target = _target(c).cuda()
    vol, nrm = _dev(c["data"]), _dev(c["nrm"])
    lut = _dev(c["lut0"], True)
    opt = torch.optim.Adam([lut], lr=0.01)
    losses = []
    for _ in range(40):
        opt.zero_grad()
        loss = ((render_views(vol, lut, c["scene"], nrm) - target) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            lut.clamp_(0.0, 1.0)
        losses.append(loss.item())
    assert losses[-1] < 0.3 * losses[0], losses
