"""bclbm: a GB300-native lattice-Boltzmann time step for BADChIMP.

The package directory is ``badchimp-cpp_gb300``; it is imported under the
name ``bclbm`` (see ``load`` in the repository's ``__graft_entry__.py``).

Submodules
  geometry  seeded sphere packs and the reference's node numbering
  lbsolver  host mirror of the reference set-up and the ``Solver`` handle
  native    ctypes binding of libbclbm.so (include/bclbm.h)
  output    the VTU output step (Output of src/io/Output.h), native writer
  serving   multi-request serving loop on one GPU
  build     nvcc build of libbclbm.so for sm_103a
"""

from . import geometry  # noqa: F401
from . import native  # noqa: F401
from . import lbsolver  # noqa: F401
from . import serving  # noqa: F401
from . import output  # noqa: F401

__all__ = ["geometry", "native", "lbsolver", "serving", "output", "build_native"]


def build_native(force: bool = False):
    from . import build as _build
    return _build.build(force=force)
