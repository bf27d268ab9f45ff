"""GB300-native GPU path tracer with the interface of SLR's PTRenderer /
VolumetricPTRenderer.  The compute path is the CUDA library
``slr_gb300/lib/libslrgpu.so`` (C ABI in ``include/slrgpu.h``)."""
from .scene_desc import SceneDesc  # noqa: F401
