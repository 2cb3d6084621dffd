"""GB300-native drop-in for Chipmunk2D's cpSpaceStep path.

The product is the C-ABI shared library ``libchipmunk_gb300.so`` built from
``csrc/`` (C host code + sm_103a CUDA kernels); ``include/chipmunk_gb300.h``
declares its entry points.  This package only locates, builds and binds it
for Python callers (tests, benchmark).
"""
from ._lib import (LIB_PATH, HEADER, bind, load_gpu_library, Scene,  # noqa: F401
                   cpVect, cpBB, cpTransform, cpShapeFilter, cpContactPointSet)
