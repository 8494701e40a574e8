"""Host-side mirror of Seismic.jl's shot-profile wave-equation migration operator
(src/Imaging/ShotProfileWEM.jl) over the GB300 C library shotwem.so.

    from wemgpu import Context, Shots, migrate, ShotProfileWEM

Arrays follow the reference's layouts: vel [nmx*nmy, nz], image [nmx*nmy, nz],
traces [ntrace, nt].
"""
from ._lib import WemError, build, lib, LIB_PATH, EXPORTS  # noqa: F401
from .api import Context, Shots, elastic, make_params, migrate, wem_dropin  # noqa: F401
