"""imsrg_gb300: the IMSRG(2) scalar commutator [X,Y] of IMSRG++ on one GB300.

The compute path is hand-written CUDA for sm_103a behind a C ABI
(include/imsrg_gb300.h, library imsrg_gb300/_build/libimsrg_gb300.so);
this package binds it with ctypes and mirrors the reference's Python
interface (ModelSpace, Operator, Commutator, BCH, Generator, IMSRGSolver).
"""

from ._lib import IMSRGError, PREC_FP64, PREC_SPLIT, lib, library_path  # noqa: F401
from .api import (BCH, Commutator, CommutatorBatch, DeviceOperator, Generator, IMSRGSolver,  # noqa: F401
                  ModelSpace, Operator, parse_reference)

__all__ = ["BCH", "Commutator", "CommutatorBatch", "DeviceOperator", "Generator", "IMSRGSolver", "ModelSpace", "Operator",
           "IMSRGError", "PREC_FP64", "PREC_SPLIT", "lib", "library_path", "parse_reference"]
