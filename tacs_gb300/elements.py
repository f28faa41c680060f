"""Element objects of the hot path, named like the reference's tacs.elements
(tacs/elements.pyx): Quad4Shell with its transforms, Element3D with
LinearElasticity3D and LinearHexaBasis, and the load elements
(Traction3D, ShellPressure from Element.createElementPressure).  They carry
data for tacs_gb300.TACS.Assembler; the GPU kernels do the element work."""
from __future__ import annotations

import numpy as np

from . import constitutive as _con


class ShellNaturalTransform:
    """TACSShellNaturalTransform (src/elements/shell/
    TACSShellElementTransform.h)."""
    kind = 0
    axis = (1.0, 0.0, 0.0)


class ShellRefAxisTransform:
    """TACSShellRefAxisTransform(axis)."""
    kind = 1

    def __init__(self, axis):
        a = np.asarray(axis, np.float64)
        self.axis = tuple(a / np.linalg.norm(a))


class ShellPressure:
    """TACSShellPressure: a uniform pressure p, or four nodal pressures."""

    def __init__(self, p):
        p = np.atleast_1d(np.asarray(p, np.float64))
        self.values = np.full(4, p[0]) if p.size == 1 else p.reshape(4)


class Quad4Shell:
    """TACSQuad4Shell(transform, con): linear MITC4 shell, 6 dof/node."""
    vars_per_node, num_nodes, elem_type = 6, 4, 0

    def __init__(self, transform, con):
        if not isinstance(con, _con.IsoShellConstitutive):
            raise NotImplementedError(
                "the GPU path implements isotropic shell constitutive data")
        self.transform = transform if transform is not None \
            else ShellNaturalTransform()
        self.con = con

    def getVarsPerNode(self):
        return 6

    def getNumNodes(self):
        return 4

    def createElementPressure(self, faceIndex, p):
        return ShellPressure(p)


class LinearHexaBasis:
    """TACSLinearHexaBasis: trilinear 8-node hexahedron."""
    num_nodes = 8


class LinearElasticity3D:
    """TACSLinearElasticity3D(con)."""

    def __init__(self, con):
        if not isinstance(con, _con.SolidConstitutive):
            raise NotImplementedError("solid elasticity needs SolidConstitutive")
        self.con = con


class Traction3D:
    """TACSTraction3D(varsPerNode, faceIndex, basis, traction): a constant
    surface traction (tx, ty, tz) on one face of a hex element."""

    def __init__(self, varsPerNode, faceIndex, basis, traction, coordComp=True):
        t = np.asarray(traction, np.float64).ravel()
        if t.size != 3:
            raise NotImplementedError("a constant 3-component traction")
        self.face, self.values = int(faceIndex), t


class Element3D:
    """TACSElement3D(model, basis): hex8 linear elasticity, 3 dof/node."""
    vars_per_node, num_nodes, elem_type = 3, 8, 1

    def __init__(self, model, basis):
        if not isinstance(model, LinearElasticity3D) or not isinstance(
                basis, LinearHexaBasis):
            raise NotImplementedError(
                "the GPU path implements LinearElasticity3D on LinearHexaBasis")
        self.model, self.basis, self.con = model, basis, model.con

    def getVarsPerNode(self):
        return 3

    def getNumNodes(self):
        return 8

    def createElementTraction(self, faceIndex, trac):
        return Traction3D(3, faceIndex, self.basis, trac)
