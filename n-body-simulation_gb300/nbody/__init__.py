"""Python side of the GB300 N-body library: ctypes binding of libnbody_cuda.so (lib), seeded
input generators in the reference's units and CSV layout (generators)."""

from . import generators  # noqa: F401
