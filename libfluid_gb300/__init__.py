"""libfluid_gb300: GB300-native PBF step + marching cubes behind libfluid's solver interface."""
from . import capi  # noqa: F401
