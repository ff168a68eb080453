"""qdfn: GB300 (sm_103a) implementation of the Quake-DFN earthquake-cycle hot path.

Host-side mirror of the reference's entry points over the C ABI of libqdfn.so:
  qdfn.geometry  ReadBulkInput / BulkToSegment / ReadSegmentInput / RotVerts_UnitVectors
  qdfn.assemble  stiffness assembly (Okada rectangles, triangular dislocations)
  qdfn.simulate  main (dense) and main_H (H-matrix), Simulation object API
  qdfn.synth     seeded synthetic fault systems for tests and benchmarks
"""
from . import _lib, build, geometry, synth  # noqa: F401
from ._lib import QdfnError, load  # noqa: F401

__version__ = "0.1.0"


def library_path():
    return _lib.lib_path()
