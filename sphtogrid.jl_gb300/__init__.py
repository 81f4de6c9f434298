"""GB300 (sm_103a) implementation of SPHtoGrid.jl's ``sphMapping`` deposition
path behind the reference's interface.

Public names mirror the Julia package: ``mappingParameters``, ``sphMapping``
and the SPHKernels kernel constructors ``Cubic``, ``Quintic``,
``WendlandC4``, ``WendlandC6``, ``WendlandC8``.  All compute runs in
``libsphgrid.so`` (CUDA); there is no CPU fallback.
"""
from ._lib import SPHtoGridError, Context, default_context  # noqa: F401
from .parameters import (Cubic, MappingParameters, Quintic, SPHKernel, WendlandC4,  # noqa: F401
                         WendlandC6, WendlandC8, kernel_from_name, mappingParameters)
from .mapping import map_it, rotation_matrix_xyz, sph_footprints, sphMapping  # noqa: F401


def __getattr__(name):
    # torch is only needed for the differentiable path
    if name in ("sph_map_differentiable", "SPHMapFunction"):
        from . import autograd
        return getattr(autograd, name)
    if name == "healpix_map":
        from . import healpix
        return healpix.healpix_map
    if name == "distributed_cic_map":
        from . import distributed
        return distributed.distributed_cic_map
    if name in ("write_fits_image", "read_fits_image", "read_allsky_fits_image",
                "write_vtk_image", "get_map_grid_2D", "get_map_grid_3D"):
        from . import io
        return getattr(io, name)
    if name == "SPHBatch" or name == "MapSpec":
        from . import batch
        return getattr(batch, name)
    raise AttributeError(name)

__all__ = ["mappingParameters", "MappingParameters", "sphMapping", "map_it", "sph_footprints", "Cubic", "Quintic",
           "WendlandC4", "WendlandC6", "WendlandC8", "SPHKernel", "kernel_from_name",
           "SPHtoGridError", "Context", "default_context"]
