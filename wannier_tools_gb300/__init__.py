"""GB300-native surface Green's functions for WannierTools' surfstat / SurfaceDOSkk path.

The compute path lives in ``libwtgpu.so`` (CUDA kernels for sm_103a behind the
C ABI of ``include/wtgpu.h``); this package builds and binds it.
"""
from ._build import build  # noqa: F401
from .api import (Engine, Model, arc_post, batch_spectrum, device_info, get_tile,  # noqa: F401
                  kpath_slab, kplane_slab, set_tile, surface_dos_kk, surfgreen_1985, surfstat,
                  surfstat_grid, surfstat_post)
from .synthetic import SurfaceModel, chain_model, make_model, random_kpoints  # noqa: F401
