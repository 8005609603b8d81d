"""Generate golden host-side vectors by importing pyvr itself.

Run with the reference tree at ``--reference PATH`` (default: the
``PYVR_REFERENCE`` environment variable).  moderngl, matplotlib, PIL and vtk are replaced by
empty import stubs: none of the functions sampled here touch them.

Writes ``tests/golden/reference_host.npz`` holding, for a set of cases:
camera position/up (float64), view and projection matrices (float32 bytes
as the reference renderer sends them), light uniforms, RenderConfig presets,
opacity/colour/RGBA LUTs, and ``compute_normal_volume`` outputs.
"""

import argparse
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _Stub(types.ModuleType):
    """Module whose every attribute is a do-nothing placeholder class."""

    def __getattr__(self, attr):
        if attr.startswith("__"):
            raise AttributeError(attr)
        return type(attr, (), {"__init__": lambda self, *a, **k: None})


class _StubFinder:
    """Import hook serving a _Stub for the absent GL / GUI / VTK packages."""

    ROOTS = ("moderngl", "matplotlib", "PIL", "vtk")

    def find_spec(self, fullname, path=None, target=None):
        import importlib.machinery
        if fullname.split(".")[0] in self.ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        mod = _Stub(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        pass


def _stub_modules():
    sys.meta_path.insert(0, _StubFinder())


CAMERA_CASES = [
    # target, azimuth, elevation, roll, distance, fov, aspect, init_pos, init_up
    ((0, 0, 0), np.pi / 4, np.pi / 6, 0.0, 3.0, np.pi / 4, 1.0, None, None),
    ((0, 0, 0), 0.0, 0.0, 0.0, 3.0, np.pi / 4, 1.0, None, None),
    ((0, 0, 0), np.pi / 2, 0.0, 0.0, 3.0, np.pi / 4, 1.0, None, None),
    ((0, 0, 0), 0.0, np.pi / 2, 0.0, 3.0, np.pi / 4, 1.0, None, None),
    ((0.1, -0.2, 0.3), 1.1, -0.4, 0.3, 2.5, np.pi / 3, 16 / 9, None, None),
    ((0, 0, 0), -2.0, 0.9, -0.7, 4.0, 0.6, 0.75, (0.0, 1.0, 0.0), (1.0, 0.0, 0.0)),
    ((0, 0, 0), 0.3, 0.2, 0.0, 3.5, np.pi / 4, 2.0, (0.0, 0.0, 2.0), (0.0, 0.0, 1.0)),
] + [((0, 0, 0), 2 * np.pi * k / 16, np.pi / 6, 0.0, 3.0, np.pi / 4, 1.0, None, None)
     for k in range(16)]

LIGHT_CASES = ["directional_c1", "default", "point", "ambient_only", "directional_z"]


def main(reference: str, out: str) -> None:
    _stub_modules()
    sys.path.insert(0, reference)
    from pyvr.camera import Camera
    from pyvr.config import RenderConfig
    from pyvr.datasets.synthetic import compute_normal_volume
    from pyvr.lighting import Light
    from pyvr.transferfunctions import ColorTransferFunction, OpacityTransferFunction

    g = {}
    # ---- cameras -----------------------------------------------------------
    cam_params, pos, up, view, proj = [], [], [], [], []
    for tgt, az, el, roll, dist, fov, aspect, ip, iu in CAMERA_CASES:
        kw = {}
        if ip is not None:
            kw["init_pos"] = np.array(ip, dtype=np.float32)
            kw["init_up"] = np.array(iu, dtype=np.float32)
        cam = Camera.from_spherical(target=np.array(tgt, dtype=np.float32), azimuth=float(az),
                                    elevation=float(el), roll=float(roll), distance=float(dist),
                                    fov=float(fov), **kw)
        p, u = cam.get_camera_vectors()
        pos.append(np.asarray(p, dtype=np.float64))
        up.append(np.asarray(u, dtype=np.float64))
        view.append(cam.get_view_matrix())
        proj.append(cam.get_projection_matrix(float(aspect)))
        ipv = (1.0, 0.0, 0.0) if ip is None else ip
        iuv = (0.0, 0.0, 1.0) if iu is None else iu
        cam_params.append([*tgt, az, el, roll, dist, fov, aspect, *ipv, *iuv])
    g["camera_params"] = np.array(cam_params, dtype=np.float64)
    g["camera_pos"] = np.stack(pos)
    g["camera_up"] = np.stack(up)
    g["camera_view"] = np.stack(view)
    g["camera_proj"] = np.stack(proj)

    # ---- lights ------------------------------------------------------------
    lights = {
        "directional_c1": Light.directional([1, -1, 0], ambient=0.2, diffuse=0.8),
        "default": Light.default(),
        "point": Light.point_light(np.array([2.0, 3.0, -1.0]), ambient=0.1, diffuse=0.7),
        "ambient_only": Light.ambient_only(0.4),
        "directional_z": Light.directional(np.array([0.0, 0.0, -2.0]), 0.3, 0.6, distance=5.0),
    }
    g["light_uniforms"] = np.array(
        [[*lights[k].position, *lights[k].target, lights[k].ambient_intensity,
          lights[k].diffuse_intensity] for k in LIGHT_CASES], dtype=np.float64)

    # ---- render configs ----------------------------------------------------
    presets = ["preview", "fast", "balanced", "high_quality", "ultra_quality"]
    g["config_presets"] = np.array(
        [[c.step_size, c.max_steps, float(c.early_ray_termination), c.opacity_threshold,
          c.reference_step_size, c.estimate_samples_per_ray()]
         for c in (getattr(RenderConfig, p)() for p in presets)], dtype=np.float64)

    # ---- transfer functions ------------------------------------------------
    otfs = [OpacityTransferFunction.linear(0.0, 0.1),
            OpacityTransferFunction.one_step(0.4, 0.05, 0.9),
            OpacityTransferFunction.peaks([0.3, 0.7], opacity=0.9, eps=0.05, base=0.1),
            OpacityTransferFunction([(0.0, 0.0), (0.3, 0.1), (0.8, 0.9), (1.0, 0.5)], lut_size=100)]
    ctfs = [ColorTransferFunction.grayscale(),
            ColorTransferFunction([(0.0, (0.0, 0.0, 0.0)), (0.5, (1.0, 0.0, 0.0)),
                                   (1.0, (1.0, 1.0, 1.0))]),
            ColorTransferFunction.two_color_ramp((0.1, 0.2, 0.3), (0.9, 0.5, 0.0), lut_size=64)]
    for i, o in enumerate(otfs):
        g[f"otf_lut_{i}"] = o.to_lut()
        g[f"otf_lut_{i}_37"] = o.to_lut(37)
    for i, c in enumerate(ctfs):
        g[f"ctf_lut_{i}"] = c.to_lut()
        g[f"ctf_lut_{i}_37"] = c.to_lut(37)

    # ---- normals -----------------------------------------------------------
    rng = np.random.default_rng(1234)
    vols = {"rand_f32": rng.random((7, 9, 11), dtype=np.float32),
            "rand_u8": rng.integers(0, 256, size=(6, 5, 8), dtype=np.uint8),
            "flat": np.full((4, 5, 6), 0.25, dtype=np.float32)}
    for k, v in vols.items():
        g[f"normals_in_{k}"] = v
        g[f"normals_out_{k}"] = compute_normal_volume(v)

    np.savez_compressed(out, **g)
    print(f"wrote {out}: {len(g)} arrays")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYVR_REFERENCE"),
                    help="path of the pyvr tree (default: $PYVR_REFERENCE)")
    ap.add_argument("--out", default=os.path.join(HERE, "reference_host.npz"))
    a = ap.parse_args()
    if not a.reference:
        ap.error("give --reference or set PYVR_REFERENCE")
    main(a.reference, a.out)
