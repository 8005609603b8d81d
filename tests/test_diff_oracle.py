"""The PyTorch-autograd reference marcher (oracle/march_torch.py) against
central finite differences of its own float64 form and against the other
oracles' images -- the checker of the differentiable path, checked on CPU."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle
from oracle import march_fp64, march_torch
from pyvr_gb300 import Camera, Light, RenderConfig, Volume, compute_normal_volume
from pyvr_gb300 import workloads as W
from pyvr_gb300.renderer import rgba_lut


def _scene(n=10, res=12, normals=True, seed=0):
    data = W.value_noise((n, n, n), seed=seed).astype(np.float32)
    vol = Volume(data=data, normals=compute_normal_volume(data) if normals else None,
                 min_bounds=np.full(3, -1.0, np.float32), max_bounds=np.full(3, 1.0, np.float32))
    rng = np.random.default_rng(seed)
    lut = rgba_lut(W.standin_colormap(seed % 12), W.random_opacity(rng, 6, 0.6), 16)
    cam = Camera.from_spherical(np.zeros(3, np.float32), 0.7, 0.4, 0.0, 3.0)
    cfg = RenderConfig(step_size=0.05, max_steps=200, reference_step_size=0.01)
    s = W.frame_inputs(vol, cam, Light.directional([1, -1, 0], 0.2, 0.8), cfg, lut, res, res)
    return s


def test_float32_form_matches_the_c_oracle():
    s = _scene()
    _, of, _ = oracle.render(s)
    img, _ = march_torch.render_view(torch.tensor(s["volume"]), torch.tensor(s["lut"]), s,
                                     torch.tensor(s["normals"]), torch.float32)
    assert np.abs(img.numpy() - of).max() < 2e-6


def test_float64_form_matches_the_fp64_oracle():
    s = _scene(normals=False)
    want, _ = march_fp64.render_fp64(s)
    img, _ = march_torch.render_view(torch.tensor(s["volume"], dtype=torch.float64),
                                     torch.tensor(s["lut"], dtype=torch.float64), s, None, torch.float64)
    assert np.abs(img.numpy() - want).max() < 1e-12


@pytest.mark.parametrize("normals", [True, False])
def test_autograd_matches_central_differences(normals):
    s = _scene(normals=normals, seed=1)
    vol = torch.tensor(s["volume"], dtype=torch.float64, requires_grad=True)
    lut = torch.tensor(s["lut"], dtype=torch.float64, requires_grad=True)
    nrm = torch.tensor(s["normals"]) if normals else None
    target = torch.rand((s["height"], s["width"], 4), dtype=torch.float64,
                        generator=torch.Generator().manual_seed(5))

    def loss(v, l):
        img, _ = march_torch.render_view(v, l, s, nrm, torch.float64)
        return ((img - target) ** 2).mean()

    loss(vol, lut).backward()
    gv, gl = vol.grad.numpy(), lut.grad.numpy()
    h = 1e-6
    picks = [("lut", np.unravel_index(i, gl.shape)) for i in np.argsort(-np.abs(gl).ravel())[:6]]
    picks += [("vol", np.unravel_index(i, gv.shape)) for i in np.argsort(-np.abs(gv).ravel())[:6]]
    for which, idx in picks:
        base_v, base_l = vol.detach().clone(), lut.detach().clone()
        plus_v, plus_l = base_v.clone(), base_l.clone()
        minus_v, minus_l = base_v.clone(), base_l.clone()
        if which == "lut":
            plus_l[idx] += h
            minus_l[idx] -= h
            g = gl[idx]
        else:
            plus_v[idx] += h
            minus_v[idx] -= h
            g = gv[idx]
        with torch.no_grad():
            fd = (loss(plus_v, plus_l) - loss(minus_v, minus_l)).item() / (2 * h)
        assert abs(fd - g) <= 1e-5 * max(abs(fd), 1e-3), (which, idx, fd, g)


def test_render_views_checks_its_inputs():
    from pyvr_gb300.diff import _check_inputs
    vol, lut = torch.zeros((4, 4, 4)), torch.zeros((16, 4))
    with pytest.raises(TypeError, match="CUDA"):
        _check_inputs(vol, lut, None)  # host tensors never reach the kernel
