"""GB300-native image-quilting hot path: a drop-in for ImageQuilting.jl's `iqsim`.

The compute runs in libiqgpu.so (hand-written CUDA for sm_103a, C ABI in include/iqgpu.h);
this package is the Python host side. Load it under any module name, e.g.

    spec = importlib.util.spec_from_file_location(
        "iqgpu", "<repo>/imagequilting.jl_gb300/__init__.py",
        submodule_search_locations=["<repo>/imagequilting.jl_gb300"])
"""
from ._lib import IQError, load  # noqa: F401
from .api import (Context, default_context, fastdistance, finddisabled, genpath,  # noqa: F401
                  graphcut, iqsim, pick, voxelreuse)
from .autotune import autotune  # noqa: F401
from .build import build  # noqa: F401
from .shard import gather_realizations, iqsim_shard, shard_range  # noqa: F401

__all__ = ["iqsim", "voxelreuse", "Context", "fastdistance", "pick", "graphcut",
           "finddisabled", "genpath", "autotune", "build", "load", "IQError", "shard_range",
           "iqsim_shard", "gather_realizations"]
