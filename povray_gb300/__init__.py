"""GB300-native trace path of POV-Ray: CUDA kernels for sm_103a behind the
C ABI in include/povgpu.h, plus the host-side block driver."""
from . import abi, scenes  # noqa: F401
from .render import GpuScene, GpuTraceTask, BlockSource  # noqa: F401
