"""GB300 (sm_103a) rasterizer for gudni's scene format.

  scene      the ShapeTree API mirror and the serializer (scene -> the reference's piles)
  raster     the generateCall replacement over the C ABI (libgudni_cuda.so)
  batch      many serialized scenes rendered in one persistent launch
  autotune   tile size and threads per tile per canvas-size bucket
  adjoint    gradients of a per-pixel L2 loss w.r.t. curve points and colours
  fit        batched fitting by Adam
  replicas   the multi-GPU (replica) timing logic
  scenes     seeded synthetic workloads
  lib, build ctypes bindings and the in-tree build of the native libraries

The raster path has no CPU fallback: without the CUDA library or a device, the entry
points raise.
"""
