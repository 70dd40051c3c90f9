"""ffip_gb300: GB300-native (sm_103a) FDTD time-stepping for ffip configs."""
from .native import FfipError, NativeSim, load, run_json, transpose  # noqa: F401
