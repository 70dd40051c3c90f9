"""ffip_gb300: GB300-native (sm_103a) FDTD time-stepping for ffip configs.

`import ffip_gb300 as ffip` gives the reference front-end's names
(Simulation, Vector3, Medium, Sphere, Box, Two_Medium_Box, Source,
Gaussian1, PML, run_until_time, Adjoint_Source, Adjoint_Volume, transpose, ...)
running in-process on the GPU; `NativeSim` / `run_json` are the lower-level
handle and one-call forms of the C ABI.
"""
from .geom import (Box, DeybeSusceptibility, DrudeSusceptibility, General_Medium_Box, GeometricObject,  # noqa: F401
                   LorentzianSusceptibility, Medium, Sphere, Susceptibility, Two_Medium_Box, Vector3, cmp_shape,
                   getgrid, metadata_to_pts, planar_polygon, sph2cart)
from .native import FfipError, NativeSim, check_inside, load, run_json, transpose  # noqa: F401
from .native import to_convolve as TO_convolve  # noqa: F401
from .native import to_convolve_transpose as TO_convolve_transpose  # noqa: F401
from .simulation import (PML, Adjoint_Flux, Adjoint_Source, Adjoint_Volume, Fields_DFT, Flux_Box,  # noqa: F401
                         Flux_Region, Geom_Info, Simulation, Symmetry, field_match_objective, run_until_dft,
                         run_until_fields_decay, run_until_time, sensitivity_scatter)
from .source import Gaussian1, Gaussian2, Inhom_Source, Source, Source_Function  # noqa: F401
