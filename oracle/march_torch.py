"""PyTorch-autograd reference marcher -- TEST INFRASTRUCTURE ONLY.

The march of pyvr/shaders/volume.frag.glsl:70-121 written with plain torch
operations on CPU tensors, so that autograd gives the gradient of the image
with respect to the LUT and the voxel values.  It is the checker of the
hand-written backward (``pvr_diff_backward``); it is never called by the
``pyvr_gb300`` package.

Two arithmetic modes:

* ``torch.float32``: ray setup from the float32 frame constants of
  ``march_ref.c`` (``oracle.frame_constants``) and every operation rounded
  to float32 in the order of the CUDA march, positions advanced by repeated
  float32 additions: the same samples as the kernel.  Lerps are a + t*(b-a)
  with two roundings (the kernel rounds once) and exp is torch.exp, so
  values agree to a few ulp;
* ``torch.float64``: everything in float64 (the central finite-difference
  reference, with ``march_fp64.py``'s ray setup).

Semantics as march_fp64.py: texel-centre trilinear sampling with
clamp-to-edge on the (D,H,W) texture read through the z/y/x swizzle
(texel (x, y, z) = flat[z + D*(y + H*x)]), two-entry LUT lerp, Beer-Lambert
opacity, Lambert shading with constant normals (a given normal volume, or
(density, 0, 0)), front-to-back compositing while alpha < 0.99, loop ended
at max_steps or when the ray has left the box.
"""

from __future__ import annotations

import numpy as np
import torch


def _setup32(scene, W, H):
    import oracle
    fc = oracle.frame_constants(scene)
    ip, iv, light_dir, inv_ext, alpha_k = fc[0:8], fc[8:20], fc[20:23], fc[23:26], fc[26]
    f32 = torch.float32
    py, px = torch.meshgrid(torch.arange(H, dtype=f32), torch.arange(W, dtype=f32), indexing="ij")
    px, py = px.reshape(-1), py.reshape(-1)
    uvx = (px + 0.5) / float(W)
    uvy = (py + 0.5) / float(H)
    nx, ny = uvx * 2.0 - 1.0, uvy * 2.0 - 1.0
    c = lambda v: torch.tensor(float(v), dtype=f32)
    ex = ((c(ip[0]) * nx + c(ip[1]) * ny) + c(ip[2]) * -1.0) + c(ip[3]) * 1.0
    ey = ((c(ip[4]) * nx + c(ip[5]) * ny) + c(ip[6]) * -1.0) + c(ip[7]) * 1.0
    w = [((c(iv[r * 4]) * ex + c(iv[r * 4 + 1]) * ey) + c(iv[r * 4 + 2]) * -1.0) + c(iv[r * 4 + 3]) * 0.0
         for r in range(3)]
    wl = 1.0 / torch.sqrt((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2])
    d = torch.stack([w[a] * wl for a in range(3)], 1)
    cam = torch.tensor(np.asarray(scene["cam_pos"], np.float32))
    bmin = torch.tensor(np.asarray(scene["bmin"], np.float32))
    bmax = torch.tensor(np.asarray(scene["bmax"], np.float32))
    with np.errstate(all="ignore"):
        inv = 1.0 / d
    t0 = (bmin - cam) * inv
    t1 = (bmax - cam) * inv
    lo, hi = torch.fmin(t0, t1), torch.fmax(t0, t1)
    tn = torch.fmax(torch.fmax(lo[:, 0], lo[:, 1]), lo[:, 2])
    tf = torch.fmin(torch.fmin(hi[:, 0], hi[:, 1]), hi[:, 2])
    hit = (tn <= tf) & (tf > 0.0)
    tn = torch.fmax(tn, torch.zeros_like(tn))
    pos = cam + d * tn[:, None]
    dstep = d * c(scene["step_size"])
    return (hit, pos, dstep, d, torch.tensor(np.asarray(inv_ext, np.float32)),
            torch.tensor(np.asarray(light_dir, np.float32)), float(alpha_k), f32)


def _setup64(scene, W, H):
    f64 = torch.float64
    ip = np.linalg.inv(np.asarray(scene["proj"], np.float64).T)
    iv = np.linalg.inv(np.asarray(scene["view"], np.float64).T)
    py, px = np.mgrid[0:H, 0:W]
    ndc = np.stack([(px.ravel() + 0.5) / W * 2 - 1, (py.ravel() + 0.5) / H * 2 - 1], 0)
    clip = np.vstack([ndc, -np.ones((1, ndc.shape[1])), np.ones((1, ndc.shape[1]))])
    eye = ip @ clip
    eye = np.vstack([eye[:2], -np.ones((1, eye.shape[1])), np.zeros((1, eye.shape[1]))])
    d = (iv @ eye)[:3].T
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    o = np.asarray(scene["cam_pos"], np.float64)
    bmin = np.asarray(scene["bmin"], np.float64)
    bmax = np.asarray(scene["bmax"], np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        t0 = (bmin - o) * inv
        t1 = (bmax - o) * inv
    tn = np.fmin(t0, t1).max(axis=1)
    tf = np.fmax(t0, t1).min(axis=1)
    hit = (tn <= tf) & (tf > 0)
    tn = np.maximum(tn, 0.0)
    pos = o + d * tn[:, None]
    lv = np.asarray(scene["light_target"], np.float64) - np.asarray(scene["light_pos"], np.float64)
    ln = np.linalg.norm(lv)
    light_dir = lv / ln if ln > 0 else np.zeros(3)
    T = lambda a: torch.tensor(np.asarray(a, np.float64), dtype=f64)
    return (T(hit).bool(), T(pos), T(d * float(scene["step_size"])), T(d), T(1.0 / (bmax - bmin)),
            T(light_dir), float(scene["step_size"]) / float(scene["reference_step_size"]), f64)


def _lerp(a, b, t):
    return a + t * (b - a)


def render_view(volume, lut, scene: dict, normals=None, dtype=torch.float32):
    """Float RGBA image (H, W, 4) of one view, differentiable in ``volume``
    ((D,H,W) tensor) and ``lut`` ((n,4) tensor), plus the per-pixel loop
    lengths.  ``scene``: the keys of ``pyvr_gb300.workloads.frame_inputs``
    (its volume/lut/normals entries are only used for the float32 frame
    constants)."""
    W, H = int(scene["width"]), int(scene["height"])
    hit, pos, dstep, d, inv_ext, light_dir, K, dt = (
        _setup32(scene, W, H) if dtype == torch.float32 else _setup64(scene, W, H))
    D, Hh, Ww = volume.shape
    ext = (Ww, Hh, D)
    fext = [torch.tensor(float(e), dtype=dt) for e in ext]
    vs = torch.tensor(float(scene.get("value_scale", 1.0)), dtype=dt)
    flat = volume.to(dt).reshape(-1)
    nflat = None if normals is None else torch.as_tensor(normals).to(dt).reshape(-1, 3).detach()
    lutd = lut.to(dt)
    nl = lutd.shape[0]
    bmin = torch.tensor(np.asarray(scene["bmin"], np.float64 if dt == torch.float64 else np.float32),
                        dtype=dt)
    amb = torch.tensor(float(scene["ambient"]), dtype=dt)
    dif = torch.tensor(float(scene["diffuse"]), dtype=dt)
    Kt = torch.tensor(K, dtype=dt)
    R = hit.shape[0]
    acc = torch.zeros((R, 4), dtype=dt)
    steps = torch.zeros(R, dtype=torch.int32)
    done = ~hit
    entered = torch.zeros(R, dtype=torch.bool)
    pos = pos.clone()
    for i in range(int(scene["max_steps"])):
        live = ~done & (acc[:, 3].detach() < 0.99)
        done = done | ~live
        if not bool(live.any()):
            break
        t = (pos - bmin) * inv_ext
        valid = live & ((t >= 0) & (t <= 1)).all(1)
        nv = t.new_zeros(R, dtype=torch.bool)
        for a in range(3):
            nv = nv | ((t[:, a] < 0) & (dstep[:, a] <= 0)) | ((t[:, a] > 1) & (dstep[:, a] >= 0))
        stop = live & ~valid & (entered | nv)
        done = done | stop
        entered = entered | valid
        steps = torch.where(live & ~stop, torch.full_like(steps, i + 1), steps)
        sel = torch.nonzero(valid).squeeze(1)
        if sel.numel():
            u = [t[sel, a] * fext[a] - 0.5 for a in range(3)]
            fl = [torch.floor(x) for x in u]
            fr = [x - f for x, f in zip(u, fl)]
            k = [f.long() for f in fl]
            lo = [k[a].clamp(0, ext[a] - 1) for a in range(3)]
            hi = [(k[a] + 1).clamp(0, ext[a] - 1) for a in range(3)]

            def tex(x, y, z):
                return (x * Hh + y) * D + z

            def tri(get):
                c00 = _lerp(get(lo[0], lo[1], lo[2]), get(lo[0], lo[1], hi[2]), fr[2])
                c01 = _lerp(get(lo[0], hi[1], lo[2]), get(lo[0], hi[1], hi[2]), fr[2])
                c10 = _lerp(get(hi[0], lo[1], lo[2]), get(hi[0], lo[1], hi[2]), fr[2])
                c11 = _lerp(get(hi[0], hi[1], lo[2]), get(hi[0], hi[1], hi[2]), fr[2])
                return _lerp(_lerp(c00, c01, fr[1]), _lerp(c10, c11, fr[1]), fr[0])

            dens = tri(lambda x, y, z: flat[tex(x, y, z)]) * vs
            lu = dens * float(nl) - 0.5
            lfl = torch.floor(lu.detach())
            la = lu - lfl
            i0 = lfl.clamp(0, nl - 1).long()
            i1 = (lfl + 1).clamp(0, nl - 1).long()
            rgba = _lerp(lutd[i0], lutd[i1], la[:, None])
            alpha = 1.0 - torch.exp(-(rgba[:, 3] * Kt))
            if nflat is not None:
                n = torch.stack([tri(lambda x, y, z, c=c: nflat[tex(x, y, z), c]) for c in range(3)], 1)
            else:
                dd = dens.detach()
                n = torch.stack([dd, torch.zeros_like(dd), torch.zeros_like(dd)], 1)
            n2 = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
            safe = torch.where(n2 > 0, n2, torch.ones_like(n2))
            # reciprocal square root rounded once (as the kernel's __frsqrt_rn)
            inv = (1.0 / torch.sqrt(safe.double())).to(dt)
            dd_ = ((n[:, 0] * inv) * light_dir[0] + (n[:, 1] * inv) * light_dir[1]) + (n[:, 2] * inv) * light_dir[2]
            di = torch.where(n2 > 0, torch.clamp(dd_, min=0.0), torch.zeros_like(dd_))
            light = amb + dif * di
            tr = 1.0 - acc[sel, 3]
            add = torch.cat([tr[:, None] * ((rgba[:, :3] * light[:, None]) * alpha[:, None]),
                             (tr * alpha)[:, None]], 1)
            acc = acc.index_add(0, sel, add)
        pos = pos + dstep
    return acc.reshape(H, W, 4), steps.reshape(H, W)


def render_views(volume, lut, scenes, normals=None, dtype=torch.float32):
    """Stacked images (V, H, W, 4) and loop lengths of several views."""
    outs = [render_view(volume, lut, s, normals, dtype) for s in scenes]
    return torch.stack([o[0] for o in outs]), torch.stack([o[1] for o in outs])
