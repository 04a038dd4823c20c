"""Foundation path-tracer pass for GB300 (sm_103a): BVH traversal, wavefront
path tracing and an online-trained radiance cache behind the C ABI of
include/fnd_rt.h. See ``foundation_gb300.rt`` for the binding."""
from .rt import (Context, FndError, HIT_DTYPE, INVALID_ID, PinnedBuffer, Scene, load)  # noqa: F401

__all__ = ["Context", "Scene", "FndError", "HIT_DTYPE", "INVALID_ID", "PinnedBuffer", "load"]
