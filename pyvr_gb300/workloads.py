"""Seeded synthetic scenes for the benchmark and test configurations.

No dataset is involved anywhere: every volume, camera and transfer function
is generated here from a seed.  Colour maps that the configurations name by
matplotlib names ("viridis", "the 12 built-ins") are replaced by clearly
labelled stand-ins -- seeded piecewise-linear RGB ramps -- because
matplotlib's tables are not available; the LUT is an input to both the
renderer and the oracle, so parity does not depend on it.
"""

from __future__ import annotations

import numpy as np

from .camera import Camera
from .config import RenderConfig
from .lighting import Light
from .transferfunctions import ColorTransferFunction, OpacityTransferFunction
from .volume import Volume, compute_normal_volume

N_STANDIN_COLORMAPS = 12


def double_sphere(n: int = 64) -> np.ndarray:
    """max over centres (+-0.4, 0, 0) of clip(1 - |p - c| / 0.5, 0, 1) on the
    grid linspace(-1, 1, n)^3, indexing 'ij' (array axis 0 = world x)."""
    g = np.linspace(-1.0, 1.0, n)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    out = np.zeros((n, n, n))
    for cx in (0.4, -0.4):
        r = np.sqrt((x - cx) ** 2 + y ** 2 + z ** 2)
        out = np.maximum(out, np.clip(1.0 - r / 0.5, 0.0, 1.0))
    return out.astype(np.float32)


def _upsample_axis(a: np.ndarray, axis: int, n: int) -> np.ndarray:
    """Linear interpolation along one axis, align-corners (end samples kept)."""
    m = a.shape[axis]
    x = np.linspace(0.0, m - 1.0, n)
    i0 = np.minimum(np.floor(x).astype(np.int64), m - 2) if m > 1 else np.zeros(n, np.int64)
    w = (x - i0) if m > 1 else np.zeros(n)
    a0 = np.take(a, i0, axis=axis)
    a1 = np.take(a, np.minimum(i0 + 1, m - 1), axis=axis)
    shape = [1] * a.ndim
    shape[axis] = n
    w = w.reshape(shape).astype(a.dtype)
    return a0 + w * (a1 - a0)


def value_noise(shape, seed: int, lattices=(8, 16, 32, 64)) -> np.ndarray:
    """4-octave value noise in [0, 1]: uniform[0,1] lattices of 8^3 .. 64^3
    from ``default_rng(seed)``, each trilinearly upsampled to ``shape``
    (align-corners), weighted 0.5^k, summed and min-max normalised."""
    rng = np.random.default_rng(seed)
    acc = np.zeros(shape, dtype=np.float32)
    for k, lat in enumerate(lattices):
        v = rng.random((lat, lat, lat), dtype=np.float32)
        for axis in range(3):
            v = _upsample_axis(v, axis, shape[axis])
        acc += np.float32(0.5 ** k) * v
    lo, hi = acc.min(), acc.max()
    return ((acc - lo) / (hi - lo)).astype(np.float32)


def standin_colormap(index: int, lut_size: int = 256) -> ColorTransferFunction:
    """Stand-in for a named matplotlib colour map: 6 seeded RGB control points."""
    rng = np.random.default_rng(7000 + int(index))
    xs = np.linspace(0.0, 1.0, 6)
    cs = rng.random((6, 3))
    return ColorTransferFunction([(float(x), tuple(map(float, c))) for x, c in zip(xs, cs)],
                                 lut_size=lut_size)


def random_opacity(rng: np.random.Generator, n_points: int, hi: float,
                   lut_size: int = 256) -> OpacityTransferFunction:
    xs = np.sort(rng.random(n_points))
    ys = rng.uniform(0.0, hi, n_points)
    return OpacityTransferFunction([(float(x), float(y)) for x, y in zip(xs, ys)],
                                   lut_size=lut_size)


def to_storage(v: np.ndarray, dtype: str) -> np.ndarray:
    """[0,1] float volume -> uint8 (round(v*255)), float16 or float32."""
    if dtype == "u8":
        return np.rint(v * 255.0).astype(np.uint8)
    if dtype == "f16":
        return v.astype(np.float16)
    return v.astype(np.float32)


# ---------------------------------------------------------------------------
# Configurations
# ---------------------------------------------------------------------------

def config_small():
    """64^3 float32 double sphere on [-1,1]^3, 256x256, balanced."""
    data = double_sphere(64)
    vol = Volume(data=data, normals=compute_normal_volume(data),
                 min_bounds=np.array([-1.0, -1.0, -1.0], np.float32),
                 max_bounds=np.array([1.0, 1.0, 1.0], np.float32))
    cam = Camera.from_spherical(target=np.zeros(3, np.float32), azimuth=np.pi / 4,
                                elevation=np.pi / 6, roll=0.0, distance=3.0, fov=np.pi / 4)
    light = Light.directional([1, -1, 0], ambient=0.2, diffuse=0.8)
    ctf = standin_colormap(0)
    otf = OpacityTransferFunction.linear(0.0, 0.1)
    return dict(volume=vol, camera=cam, light=light, ctf=ctf, otf=otf,
                config=RenderConfig.balanced(), width=256, height=256, value_scale=1.0)


def config_scale_volume(n: int = 256, seed: int = 0) -> np.ndarray:
    return value_noise((n, n, n), seed)


def config_scale(dtype: str = "f32", n: int = 256, res: int = 1024, noise=None):
    """256^3 value noise (seed 0) in u8/f16/f32, 16 orbit cameras, 1024^2,
    high_quality, 8 seeded opacity points in [0, 0.3] + stand-in colour."""
    v = config_scale_volume(n) if noise is None else noise
    data = to_storage(v, dtype)
    # normals by central differences of the stored values, as pyvr computes them
    normals = compute_normal_volume(data)
    vol = Volume(data=data, normals=normals,
                 min_bounds=np.array([-1.0, -1.0, -1.0], np.float32),
                 max_bounds=np.array([1.0, 1.0, 1.0], np.float32))
    cams = [Camera.from_spherical(target=np.zeros(3, np.float32), azimuth=2 * np.pi * k / 16,
                                  elevation=np.pi / 6, roll=0.0, distance=3.0)
            for k in range(16)]
    otf = random_opacity(np.random.default_rng(0), 8, 0.3)
    return dict(volume=vol, cameras=cams, light=Light.directional([1, -1, 0], 0.2, 0.8),
                ctf=standin_colormap(0), otf=otf, config=RenderConfig.high_quality(),
                width=res, height=res, value_scale=(1.0 / 255.0 if dtype == "u8" else 1.0))


def frame_inputs(volume: Volume, camera, light, config, lut: np.ndarray, width: int,
                 height: int, value_scale: float = 1.0, batch_camera: bool = False) -> dict:
    """Everything one frame depends on, as the uniforms/textures the reference
    renderer would set (renderer.py:107-172, 303-316), in a plain dict.
    batch_camera: camera matrices as the batch path computes them (native
    double-precision setup) instead of the ``Camera`` methods'."""
    if batch_camera:
        from .batch import job_camera_uniforms as uniforms
    else:
        from .renderer import camera_uniforms as uniforms
    view, proj, pos = uniforms(camera, width, height)
    return dict(width=width, height=height, view=view, proj=proj, cam_pos=pos,
                volume=volume.data, normals=volume.normals, value_scale=value_scale,
                bmin=volume.min_bounds, bmax=volume.max_bounds, lut=lut,
                step_size=config.step_size, reference_step_size=config.reference_step_size,
                max_steps=config.max_steps, light_pos=light.position, light_target=light.target,
                ambient=light.ambient_intensity, diffuse=light.diffuse_intensity)


def config_batching(n: int = 64, max_dim: int = 384, resolutions=(128, 256, 512, 1024), noise=None):
    """n uneven renders: per instance i (seed i) volume extents drawn
    log-uniformly from 32..max_dim per axis (non-cubic), storage uniform over
    uint8/float16/float32, value noise, resolution uniform over the given
    squares, a random camera on a sphere of radius 2.5-4 around the box, and
    a random TF (4-12 opacity points, one of the 12 stand-in colour maps).
    Normals are left to the device (numpy.gradient semantics).  noise:
    the value-noise generator (shape, seed) -> array (default value_noise)."""
    noise = noise or value_noise
    scenes = []
    for i in range(n):
        rng = np.random.default_rng(i)
        dims = tuple(int(round(x)) for x in np.exp(rng.uniform(np.log(32), np.log(max_dim), 3)))
        dtype = ["u8", "f16", "f32"][int(rng.integers(0, 3))]
        res = int(resolutions[int(rng.integers(0, len(resolutions)))])
        radius = float(rng.uniform(2.5, 4.0))
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        az = float(np.arctan2(v[1], v[0]))
        el = float(np.arcsin(np.clip(v[2], -1, 1)))
        otf = random_opacity(rng, int(rng.integers(4, 13)), 0.3)
        ctf = standin_colormap(int(rng.integers(0, N_STANDIN_COLORMAPS)))
        data = to_storage(noise(dims, i), dtype)
        vol = Volume(data=data, min_bounds=np.array([-1.0, -1.0, -1.0], np.float32),
                     max_bounds=np.array([1.0, 1.0, 1.0], np.float32))
        cam = Camera.from_spherical(target=np.zeros(3, np.float32), azimuth=az, elevation=el, roll=0.0,
                                    distance=radius)
        scenes.append(dict(volume=vol, dtype=dtype, value_scale=(1.0 / 255.0 if dtype == "u8" else 1.0),
                           camera=cam, light=Light.directional([1, -1, 0], 0.2, 0.8), ctf=ctf, otf=otf,
                           config=RenderConfig.balanced(), width=res, height=res))
    return scenes


# ---------------------------------------------------------------------------
# Serving workload
# ---------------------------------------------------------------------------

def value_noise_device(n, seed: int, dtype: str = "f32") -> np.ndarray:
    """value_noise(shape, seed) (shape = n or (n, n, n)) by the same definition
    (lattices from default_rng(seed), align-corners trilinear upsampling,
    weights 0.5^k, min-max normalisation), upsampled on the GPU for speed;
    float rounding may differ from value_noise in the last bits.  dtype: the
    storage of the result ("f32", or "u8" / "f16" as ``to_storage`` makes
    them, converted on the GPU)."""
    import torch
    import torch.nn.functional as F
    shape = (n, n, n) if isinstance(n, (int, np.integer)) else tuple(int(x) for x in n)
    rng = np.random.default_rng(seed)
    acc = torch.zeros(shape, dtype=torch.float32, device="cuda")
    for k, lat in enumerate((8, 16, 32, 64)):
        v = torch.from_numpy(rng.random((lat, lat, lat), dtype=np.float32)).cuda()
        up = F.interpolate(v[None, None], size=shape, mode="trilinear", align_corners=True)[0, 0]
        acc += (0.5 ** k) * up
        del up
    lo, hi = acc.min(), acc.max()
    acc = (acc - lo) / (hi - lo)
    if dtype == "u8":
        # round half to even, as numpy's rint
        return torch.round(acc * 255.0).to(torch.uint8).cpu().numpy()
    if dtype == "f16":
        return acc.to(torch.float16).cpu().numpy()
    return acc.cpu().numpy()


class _LazyVolumes:
    """The workload's volumes as (Volume, value_scale), generated on first
    use (``materialize`` generates them all)."""

    def __init__(self, specs, generator):
        self._specs = specs  # (extent, storage, seed)
        self._gen = generator
        self._cache = {}

    def __len__(self):
        return len(self._specs)

    def __getitem__(self, i):
        if i < 0:
            i += len(self._specs)
        if i not in self._cache:
            n, dtype, seed = self._specs[i]
            data = self._gen(n, seed, dtype)
            vol = Volume(data=data, min_bounds=np.array([-1.0, -1.0, -1.0], np.float32),
                         max_bounds=np.array([1.0, 1.0, 1.0], np.float32))
            self._cache[i] = (vol, 1.0 / 255.0 if dtype == "u8" else 1.0)
        return self._cache[i]

    def __iter__(self):
        return (self[i] for i in range(len(self)))

    def ref(self, i) -> "_VolumeRef":
        """A stand-in for volume i that generates it on first use."""
        return _VolumeRef(self, i)

    def value_scale(self, i) -> float:
        return 1.0 / 255.0 if self._specs[i][1] == "u8" else 1.0

    def extent(self, i) -> int:
        return self._specs[i][0]

    def storage(self, i) -> str:
        return self._specs[i][1]

    def materialize(self) -> None:
        for i in range(len(self)):
            self[i]


class _VolumeRef:
    """Volume i of a _LazyVolumes: the Volume's attributes, generated on first
    access (a request stream can name volumes it never makes anyone read)."""

    def __init__(self, volumes, i):
        self._volumes, self._i = volumes, i

    def resolve(self) -> Volume:
        return self._volumes[self._i][0]

    data = property(lambda self: self.resolve().data)
    normals = property(lambda self: self.resolve().normals)
    min_bounds = property(lambda self: self.resolve().min_bounds)
    max_bounds = property(lambda self: self.resolve().max_bounds)


def _storage_generator(gen):
    """A (n, seed) -> float volume generator as (n, seed, dtype) -> storage."""
    return lambda n, seed, dtype: to_storage(gen(n, seed), dtype)


class ServingWorkload:
    """Seeded serving scenario: a catalog of resident volumes (cubic, extents
    log-uniform in [min_dim, max_dim], uint8 or float16 value noise, normals
    computed on the device), per-volume camera/TF sessions, and Poisson
    request streams with the mix 70% orbit re-renders (azimuth/elevation
    deltas ~N(0, 0.05) rad, 512^2), 20% TF edits (1-3 opacity points moved by
    ~N(0, 0.05), then a 512^2 render), 5% high-quality 1024^2 captures, 5%
    new-volume loads (a volume not in the catalog replaces a catalog slot:
    uploaded, laid out with device normals, then rendered at 512^2).

    The n_extra volumes outside the catalog are the clients' pool of new
    volumes; a load brings the one that has been out of the catalog longest,
    so with a pool larger than what the byte budget holds, every load uploads
    a volume that is not resident.  Volume data is generated on first use
    (``volumes.materialize()`` generates it all up front)."""

    def __init__(self, n_volumes: int = 32, n_extra: int = 16, min_dim: int = 128,
                 max_dim: int = 512, seed: int = 0, res: int = 512, capture_res: int = 1024,
                 generator=None):
        self.res, self.capture_res = res, capture_res
        self.light = Light.directional([1, -1, 0], 0.2, 0.8)
        rng = np.random.default_rng(seed)
        specs = []
        for i in range(n_volumes + n_extra):
            n = int(round(np.exp(rng.uniform(np.log(min_dim), np.log(max_dim)))))
            dtype = "u8" if rng.random() < 0.5 else "f16"
            specs.append((n, dtype, 5000 + i))
        gen = value_noise_device if generator is None else _storage_generator(generator)
        self.volumes = _LazyVolumes(specs, gen)
        self.n_catalog = n_volumes
        self.catalog = list(range(n_volumes))  # catalog slot -> volume index
        # volumes out of the catalog, the longest-out first
        self.outside = list(range(n_volumes, n_volumes + n_extra))
        self.sessions = []
        for i in range(n_volumes + n_extra):
            srng = np.random.default_rng(9000 + i)
            self.sessions.append({
                "az": float(srng.uniform(-np.pi, np.pi)), "el": float(srng.uniform(-0.8, 0.8)),
                "dist": float(srng.uniform(2.5, 4.0)),
                "otf": [(float(x), float(y)) for x, y in zip(np.sort(srng.random(6)),
                                                            srng.uniform(0.0, 0.3, 6))],
                "ctf": standin_colormap(int(srng.integers(0, N_STANDIN_COLORMAPS)))})

    def snapshot(self):
        """The evolving state (catalog, volumes outside it, session cameras and
        opacity points), to restart request streams from the same point with
        ``restore``."""
        return (list(self.catalog), list(self.outside), [dict(s, otf=list(s["otf"])) for s in self.sessions])

    def restore(self, snap) -> None:
        catalog, outside, sessions = snap
        self.catalog = list(catalog)
        self.outside = list(outside)
        self.sessions = [dict(s, otf=list(s["otf"])) for s in sessions]

    def camera(self, vidx: int) -> Camera:
        s = self.sessions[vidx]
        return Camera.from_spherical(target=np.zeros(3, np.float32), azimuth=s["az"],
                                     elevation=s["el"], roll=0.0, distance=s["dist"])

    def requests(self, rate: float, duration: float, seed: int):
        """[(arrival offset s, kwargs of RenderRequest)] for a Poisson stream."""
        rng = np.random.default_rng(seed)
        t, out = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t >= duration:
                return out
            u = rng.random()
            slot = int(rng.integers(0, self.n_catalog))
            kind, w, cfg = "render", self.res, RenderConfig.balanced()
            if u < 0.70:
                tag = "orbit"
            elif u < 0.90:
                tag = "tf_edit"
            elif u < 0.95:
                tag, w, cfg = "capture", self.capture_res, RenderConfig.high_quality()
            else:
                tag, kind = "load", "load"
                # the volume out of the catalog longest replaces a catalog slot
                if self.outside:
                    self.outside.append(self.catalog[slot])
                    self.catalog[slot] = self.outside.pop(0)
            vidx = self.catalog[slot]
            s = self.sessions[vidx]
            if tag == "orbit":
                s["az"] += float(rng.normal(0.0, 0.05))
                s["el"] = float(np.clip(s["el"] + rng.normal(0.0, 0.05), -1.5, 1.5))
            elif tag == "tf_edit":
                pts = list(s["otf"])
                for k in rng.choice(len(pts), size=int(rng.integers(1, 4)), replace=False):
                    x, y = pts[k]
                    pts[k] = (float(np.clip(x + rng.normal(0, 0.05), 0, 1)),
                              float(np.clip(y + rng.normal(0, 0.05), 0, 1)))
                s["otf"] = sorted(pts)
            out.append((t, dict(kind=kind, volume_id=vidx, camera=self.camera(vidx), light=self.light,
                                config=cfg, color_tf=s["ctf"],
                                opacity_tf=OpacityTransferFunction(list(s["otf"])), width=w, height=w,
                                value_scale=self.volumes.value_scale(vidx), volume=self.volumes.ref(vidx),
                                tag=tag)))
