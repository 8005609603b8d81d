"""FP64 NumPy ray marcher -- TEST INFRASTRUCTURE ONLY (the float-image oracle).

Same semantics as pyvr/shaders/volume.frag.glsl:70-121 and the GL state of
pyvr/moderngl_renderer/manager.py (texel-centre trilinear sampling with
clamp-to-edge on the (D,H,W)-sized texture read through the z/y/x swizzle,
two-entry LUT lerp, Beer-Lambert opacity, Lambert shading, front-to-back
compositing stopped at alpha 0.99), evaluated in float64 for all rays in
lock-step.  It gives the error statistics of the float32 image; the exact
RGBA8 oracle is march_ref.c.
"""

from __future__ import annotations

import numpy as np


def _gl_inverse(m32: np.ndarray) -> np.ndarray:
    """Inverse of the matrix GL reads from these row-major numpy bytes."""
    return np.linalg.inv(np.asarray(m32, dtype=np.float64).T)


def _trilinear(grid: np.ndarray, ext, u):
    """grid indexed [x, y, z(, c)]; u = (ux, uy, uz) continuous texel coords."""
    i0, f = [], []
    for a in range(3):
        fl = np.floor(u[a])
        f.append(u[a] - fl)
        i0.append(fl.astype(np.int64))
    idx = [(np.clip(i0[a], 0, ext[a] - 1), np.clip(i0[a] + 1, 0, ext[a] - 1)) for a in range(3)]
    out = 0.0
    for xi in (0, 1):
        wx = f[0] if xi else 1.0 - f[0]
        for yi in (0, 1):
            wy = f[1] if yi else 1.0 - f[1]
            for zi in (0, 1):
                wz = f[2] if zi else 1.0 - f[2]
                w = wx * wy * wz
                v = grid[idx[0][xi], idx[1][yi], idx[2][zi]]
                out = out + (w[:, None] * v if v.ndim == 2 else w * v)
    return out


def render_fp64(scene: dict):
    """Float RGBA image (H, W, 4) float64 and the per-pixel in-box sample count.

    ``scene`` keys: width, height, view, proj, cam_pos, volume (D,H,W),
    value_scale, normals (D,H,W,3) or None, bmin, bmax, lut (n,4), step_size,
    reference_step_size, max_steps, light_pos, light_target, ambient, diffuse.
    """
    W, H = scene["width"], scene["height"]
    vol = np.asarray(scene["volume"])
    D, Hh, Ww = vol.shape
    flat = vol.astype(np.float64).reshape(-1) * float(scene.get("value_scale", 1.0))
    # The texture of size (D,H,W) is read as grid[x, y, z] = flat[z + D*(y + H*x)].
    grid = flat.reshape(Ww, Hh, D)
    ext = (Ww, Hh, D)
    nrm = scene.get("normals")
    ngrid = None if nrm is None else np.asarray(nrm, np.float64).reshape(Ww, Hh, D, 3)
    lut = np.asarray(scene["lut"], dtype=np.float64)
    nl = lut.shape[0]
    bmin = np.asarray(scene["bmin"], np.float64)
    bmax = np.asarray(scene["bmax"], np.float64)
    ext_w = bmax - bmin

    ip = _gl_inverse(scene["proj"])
    iv = _gl_inverse(scene["view"])
    py, px = np.mgrid[0:H, 0:W]
    ndc = np.stack([(px.ravel() + 0.5) / W * 2 - 1, (py.ravel() + 0.5) / H * 2 - 1], 0)
    clip = np.vstack([ndc, -np.ones((1, ndc.shape[1])), np.ones((1, ndc.shape[1]))])
    eye = ip @ clip
    eye = np.vstack([eye[:2], -np.ones((1, eye.shape[1])), np.zeros((1, eye.shape[1]))])
    d = (iv @ eye)[:3].T
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    o = np.asarray(scene["cam_pos"], np.float64)

    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        t0 = (bmin - o) * inv
        t1 = (bmax - o) * inv
    lo = np.fmin(t0, t1)
    hi = np.fmax(t0, t1)
    tn = lo.max(axis=1)
    tf = hi.min(axis=1)
    hit = (tn <= tf) & (tf > 0)
    tn = np.maximum(tn, 0.0)

    n = d.shape[0]
    acc = np.zeros((n, 4))
    samples = np.zeros(n, dtype=np.int64)
    pos = o + d * tn[:, None]
    step = float(scene["step_size"])
    k = step / float(scene["reference_step_size"])
    lv = np.asarray(scene["light_target"], np.float64) - np.asarray(scene["light_pos"], np.float64)
    ln = np.linalg.norm(lv)
    L = lv / ln if ln > 0 else np.zeros(3)
    amb, dif = float(scene["ambient"]), float(scene["diffuse"])
    active = hit.copy()
    for _ in range(int(scene["max_steps"])):
        active &= acc[:, 3] < 0.99
        if not active.any():
            break
        t = (pos - bmin) / ext_w
        valid = active & np.all((t >= 0) & (t <= 1), axis=1)
        sel = np.nonzero(valid)[0]
        if sel.size:
            samples[sel] += 1
            u = [t[sel, a] * ext[a] - 0.5 for a in range(3)]
            dens = _trilinear(grid, ext, u)
            lu = dens * nl - 0.5
            l0 = np.floor(lu)
            la = lu - l0
            i0 = np.clip(l0, 0, nl - 1).astype(np.int64)
            i1 = np.clip(l0 + 1, 0, nl - 1).astype(np.int64)
            rgba = lut[i0] + la[:, None] * (lut[i1] - lut[i0])
            alpha = 1.0 - np.exp(-rgba[:, 3] * k)
            if ngrid is not None:
                nv = _trilinear(ngrid, ext, u)
            else:
                nv = np.stack([dens, np.zeros_like(dens), np.zeros_like(dens)], 1)
            nn = np.linalg.norm(nv, axis=1)
            with np.errstate(invalid="ignore", divide="ignore"):
                di = np.where(nn > 0, np.maximum((nv @ L) / np.where(nn > 0, nn, 1), 0.0), 0.0)
            light = amb + dif * di
            tr = 1.0 - acc[sel, 3]
            acc[sel, :3] += (tr * alpha * light)[:, None] * rgba[:, :3]
            acc[sel, 3] += tr * alpha
        pos = pos + d * step
    return acc.reshape(H, W, 4), samples.reshape(H, W)


def blend_rgba8(img: np.ndarray) -> np.ndarray:
    """GL SRC_ALPHA/ONE_MINUS_SRC_ALPHA over a cleared UNORM8 target."""
    a = np.clip(img[..., 3], 0, 1)
    out = np.empty(img.shape, dtype=np.uint8)
    out[..., :3] = np.rint(np.clip(img[..., :3], 0, 1) * a[..., None] * 255)
    out[..., 3] = np.rint(a * a * 255)
    return out
