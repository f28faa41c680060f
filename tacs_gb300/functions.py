"""Structural functions of the hot path, named like the reference's
tacs.functions (tacs/functions.pyx): Compliance (TACSCompliance) and
KSFailure (TACSKSFailure, continuous KS aggregation)."""
from __future__ import annotations

from . import _lib


class Compliance:
    """TACSCompliance(assembler): integral of the strain energy density."""
    kind = _lib.FUNC_COMPLIANCE

    def __init__(self, assembler):
        self.assembler = assembler


class KSFailure:
    """TACSKSFailure(assembler, ksWeight, alpha, safetyFactor): continuous KS
    aggregate of the failure index (default weight 80 as in the reference)."""
    kind = _lib.FUNC_KS_FAILURE

    def __init__(self, assembler, ksWeight=80.0, alpha=1.0, safetyFactor=1.0):
        if safetyFactor != 1.0:
            raise NotImplementedError("safetyFactor != 1 is not on the GPU path")
        self.assembler, self.ksWeight = assembler, float(ksWeight)
