"""GB300-native (sm_103a) vertex-merging caustics renderer, a drop-in for the
RealCausticsEngine DLL's init()/main() path.

Layout:
  csrc/        CUDA kernels (traversal, light/camera passes, KD-tree, gather) and the
               C ABI (rc_abi.cpp) - built into librealcaustics.so
  scene.py     scene description and its Blender-layout encoding for init()
  scenes.py    seeded synthetic workloads
  session.py   Python host over the C ABI (what the Blender add-on does via ctypes)
  build.py     in-tree nvcc build
"""
from .scene import Camera, InitArgs, Light, Material, Mesh, Scene, look_at_camera  # noqa: F401

__all__ = ["Camera", "InitArgs", "Light", "Material", "Mesh", "Scene", "look_at_camera"]
