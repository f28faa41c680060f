"""Constitutive objects of the hot path, named and parameterised like the
reference's tacs.constitutive (tacs/constitutive.pyx): MaterialProperties,
IsoShellConstitutive and SolidConstitutive.  They only carry data; the
GPU kernels evaluate the constitutive relations (TACSIsoShellConstitutive,
TACSSolidConstitutive with the element scale t)."""
from __future__ import annotations


class MaterialProperties:
    """TACSMaterialProperties for an isotropic material
    (src/constitutive/TACSMaterialProperties.cpp); ys is the yield stress
    used by the von Mises failure criterion."""

    def __init__(self, rho=2700.0, specific_heat=0.0, E=70e9, nu=0.3,
                 ys=3e8, alpha=0.0, kappa=0.0, **kwargs):
        self.rho, self.E, self.nu, self.ys = float(rho), float(E), float(nu), \
            float(ys)

    def getMaterialProperties(self):
        return {"rho": self.rho, "E": self.E, "nu": self.nu, "ys": self.ys}


class IsoShellConstitutive:
    """TACSIsoShellConstitutive(props, t, tNum, tlb, tub): thickness t,
    design-variable number tNum (-1: fixed thickness)."""

    def __init__(self, props, t=1.0, tNum=-1, tlb=0.0, tub=10.0, tOffset=0.0):
        if tOffset != 0.0:
            raise NotImplementedError("shell offsets are not on the GPU path")
        self.props, self.t, self.tNum = props, float(t), int(tNum)


class SolidConstitutive:
    """TACSSolidConstitutive(props, t, tNum, tlb, tub): the stiffness is
    scaled by t (e.g. t = rho^3 for SIMP), design variable tNum."""

    def __init__(self, props, t=1.0, tNum=-1, tlb=0.0, tub=10.0):
        self.props, self.t, self.tNum = props, float(t), int(tNum)
