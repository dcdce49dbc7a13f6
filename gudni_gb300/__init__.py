"""GB300 (sm_103a) rasterizer for gudni's scene format: serializer front end, C-ABI
CUDA raster kernels and the host-side mirror of the reference interface."""
