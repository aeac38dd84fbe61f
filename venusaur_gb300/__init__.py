"""Venusaur-GB300: a GB300-native (sm_103a) path tracer for the Ray Tracing in
One Weekend sphere scene, behind the reference's Renderer / Scene / Camera /
Material / Sphere interface.  All compute runs in libvenusaur_gb300.so
(include/venu.h); this package is the host-side mirror of the interface."""
from ._lib import CAMERA_DTYPE, NODE_DTYPE, SPHERE_DTYPE, VenuError, lib  # noqa: F401
from .core import (  # noqa: F401
    Batch,
    Camera,
    CUDAOutputBuffer,
    DeviceScene,
    Material,
    Renderer,
    Scene,
    Server,
    Sphere,
    Wavefront,
    generate_random,
    generate_rtiow,
    new_accum,
    sm_count,
    write_pfm,
    write_ppm,
)

__all__ = [
    "Batch", "Camera", "CUDAOutputBuffer", "DeviceScene", "Material", "Renderer", "Scene", "Server", "Sphere",
    "Wavefront", "VenuError", "generate_random", "generate_rtiow", "new_accum", "sm_count", "write_pfm", "write_ppm", "lib",
    "SPHERE_DTYPE", "CAMERA_DTYPE", "NODE_DTYPE",
]
