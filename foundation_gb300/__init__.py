"""Foundation path-tracer pass for GB300 (sm_103a): BVH traversal, wavefront
path tracing and an online-trained radiance cache behind the C ABI of
include/fnd_rt.h. See ``foundation_gb300.rt`` for the binding."""
from .rt import (Batch, Context, FndError, HIT_DTYPE, INVALID_ID, LIGHT_DTYPE, MATERIAL_DTYPE, PinnedBuffer,  # noqa
                 InstanceScene, QUERY_ANY, QUERY_CLOSEST, Scene, TONEMAP_ACES, TONEMAP_CLAMP, TONEMAP_REINHARD, load)

__all__ = ["Batch", "Context", "InstanceScene", "Scene", "FndError", "HIT_DTYPE", "INVALID_ID", "LIGHT_DTYPE", "MATERIAL_DTYPE",
           "PinnedBuffer", "QUERY_ANY", "QUERY_CLOSEST", "TONEMAP_ACES", "TONEMAP_CLAMP", "TONEMAP_REINHARD", "load"]
