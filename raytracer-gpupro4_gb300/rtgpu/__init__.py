"""GB300 (sm_103a) LBVH ray-tracing core: Python binding of the C ABI.

The kernels live in librtgb300.so (built by rtgpu.build); this package only
binds them (rtgpu._lib), mirrors the reference's stage API (rtgpu.api) and
generates the seeded synthetic scenes (rtgpu.scenes).
"""
