"""GB300-native melt_IBM fluid RK3 substep.

The product is ``libmibm.so`` (CUDA C++ for sm_103a, C-ABI in
include/mibm.h).  This package holds the Python host mirror of the reference
interface: the ctypes binding (:mod:`abi`), the Fortran-layout case state
(:mod:`case`), mesh input (:mod:`mesh`), seeded synthetic fields
(:mod:`fields`) and the library build (:mod:`build`).
"""
from . import abi  # noqa: F401
