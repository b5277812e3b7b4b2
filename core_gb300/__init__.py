"""GB300-native estimate-and-mark pass of PUMI (SCOREC/core).

SPR gradient recovery, the SPR size field, metric edge lengths, mean-ratio
quality and split/collapse edge marking, as sm_103a CUDA kernels behind the
C ABI in include/spr_gb300.h.  This package is the Python host layer over
that library (libsprgb300.so, built by ``python -m core_gb300.build``).
"""
from ._lib import SprgError, load  # noqa: F401
from .api import Context, SizeField, apply_marks, max_iterations_for_length, mesh_delta  # noqa: F401
from .mesh import Mesh, makeMdsBox, box_counts  # noqa: F401
