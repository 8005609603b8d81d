"""pyvr_gb300: GB300 (sm_103a) CUDA ray marcher behind pyvr's VolumeRenderer API.

``from pyvr_gb300 import VolumeRenderer`` gives a renderer with the methods of
pyvr.moderngl_renderer.VolumeRenderer (load_volume, set_camera, set_light,
set_transfer_functions, set_config, render -> RGBA8 bytes).  The scene value
objects mirror pyvr's: Camera, Light, RenderConfig, Volume and the
colour/opacity transfer functions.
"""

from .camera import Camera, CameraError, get_camera_pos, get_camera_pos_from_params
from .config import RenderConfig
from .lighting import Light, LightError
from .renderer import CudaVolumeRenderer, ModernGLVolumeRenderer, VolumeRenderer
from .transferfunctions import (ColorTransferFunction, InvalidControlPointError,
                                OpacityTransferFunction, TransferFunctionError)
from .volume import Volume, VolumeError, compute_normal_volume

__version__ = "0.1.0"

__all__ = [
    "Camera", "CameraError", "get_camera_pos", "get_camera_pos_from_params", "RenderConfig",
    "Light", "LightError", "CudaVolumeRenderer", "ModernGLVolumeRenderer", "VolumeRenderer",
    "ColorTransferFunction", "OpacityTransferFunction", "TransferFunctionError",
    "InvalidControlPointError", "Volume", "VolumeError", "compute_normal_volume",
]
