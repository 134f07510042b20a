"""CPU oracle (test infrastructure only): see mibm_oracle.cpp."""
from .build import LIB, build  # noqa: F401
