"""Gate matrices and the kernel operands derived from them.

``Matrices`` gives the textbook matrices in qibo's conventions (the matrices qibojit
receives from qibo's ``NumpyMatrices``; qibo itself is not a dependency of this
engine): RZ(t) = diag(e^{-it/2}, e^{it/2}), U1(t) = diag(1, e^{it}),
U3(t, p, l) = [[e^{-i(p+l)/2} cos(t/2), -e^{-i(p-l)/2} sin(t/2)],
[e^{i(p-l)/2} sin(t/2), e^{i(p+l)/2} cos(t/2)]], fSim(t, p) acting as
[[cos t, -i sin t], [-i sin t, cos t]] on |01>, |10> and e^{-ip} on |11>.

``CustomMatrices`` restates qibojit's operand encoding
(``src/qibojit/backends/matrices.py:7-70``): controlled gates pass only the 2x2 of
their target, U1/CU1 pass the scalar e^{it}, CZ/CCZ pass Z (applied by the
"apply_z" kernel), fSim/GeneralizedfSim pass 5 scalars, DEUTSCH passes 1j*RX(2t).
"""
from __future__ import annotations

import numpy as np


class Matrices:
    def __init__(self, dtype: str = "complex128"):
        self.dtype = dtype

    def _cast(self, x):
        return np.asarray(x, dtype=self.dtype)

    # --- fixed one-qubit gates
    @property
    def H(self):
        return self._cast(np.array([[1, 1], [1, -1]]) / np.sqrt(2))

    @property
    def X(self):
        return self._cast([[0, 1], [1, 0]])

    @property
    def Y(self):
        return self._cast([[0, -1j], [1j, 0]])

    @property
    def Z(self):
        return self._cast([[1, 0], [0, -1]])

    @property
    def SX(self):
        return self._cast(0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]))

    @property
    def SXDG(self):
        return np.conj(self.SX)

    @property
    def S(self):
        return self._cast([[1, 0], [0, 1j]])

    @property
    def SDG(self):
        return self._cast([[1, 0], [0, -1j]])

    @property
    def T(self):
        return self._cast([[1, 0], [0, np.exp(1j * np.pi / 4)]])

    @property
    def TDG(self):
        return self._cast([[1, 0], [0, np.exp(-1j * np.pi / 4)]])

    def I(self, n=2):
        return self._cast(np.eye(n))

    # --- parametrised one-qubit gates
    def RX(self, theta):
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        return self._cast([[c, -1j * s], [-1j * s, c]])

    def RY(self, theta):
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        return self._cast([[c, -s], [s, c]])

    def RZ(self, theta):
        return self._cast([[np.exp(-0.5j * theta), 0], [0, np.exp(0.5j * theta)]])

    def U1(self, theta):
        return self._cast([[1, 0], [0, np.exp(1j * theta)]])

    def U2(self, phi, lam):
        ep, em = np.exp(0.5j * (phi + lam)), np.exp(0.5j * (phi - lam))
        return self._cast(np.array([[np.conj(ep), -np.conj(em)], [em, ep]]) / np.sqrt(2))

    def U3(self, theta, phi, lam):
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        ep, em = np.exp(0.5j * (phi + lam)), np.exp(0.5j * (phi - lam))
        return self._cast([[np.conj(ep) * c, -np.conj(em) * s], [em * s, ep * c]])

    # --- controlled gates as full matrices (control = first qubit)
    @staticmethod
    def _controlled(u):
        d = u.shape[0]
        out = np.eye(2 * d, dtype=u.dtype)
        out[d:, d:] = u
        return out

    @property
    def CNOT(self):
        return self._controlled(self.X)

    @property
    def CZ(self):
        return self._controlled(self.Z)

    @property
    def CY(self):
        return self._controlled(self.Y)

    @property
    def CH(self):
        return self._controlled(self.H)

    @property
    def CSX(self):
        return self._controlled(self.SX)

    @property
    def CSXDG(self):
        return self._controlled(self.SXDG)

    def CRX(self, theta):
        return self._controlled(self.RX(theta))

    def CRY(self, theta):
        return self._controlled(self.RY(theta))

    def CRZ(self, theta):
        return self._controlled(self.RZ(theta))

    def CU1(self, theta):
        return self._controlled(self.U1(theta))

    def CU2(self, phi, lam):
        return self._controlled(self.U2(phi, lam))

    def CU3(self, theta, phi, lam):
        return self._controlled(self.U3(theta, phi, lam))

    @property
    def SWAP(self):
        return self._cast([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]])

    def fSim(self, theta, phi):
        c, s = np.cos(theta), np.sin(theta)
        return self._cast([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [0, 0, 0, np.exp(-1j * phi)]])

    def GeneralizedfSim(self, u, phi):
        m = np.eye(4, dtype=complex)
        m[1:3, 1:3] = np.asarray(u)
        m[3, 3] = np.exp(-1j * phi)
        return self._cast(m)

    @property
    def TOFFOLI(self):
        return self._controlled(self.CNOT)

    @property
    def CCZ(self):
        return self._controlled(self.CZ)

    def DEUTSCH(self, theta):
        return self._controlled(self._controlled(1j * self.RX(2 * theta)))

    def Unitary(self, u):
        return self._cast(u)


class CustomMatrices(Matrices):
    """Kernel operands (qibojit backends/matrices.py:7-70)."""

    def CRX(self, theta):
        return self.RX(theta)

    def CRY(self, theta):
        return self.RY(theta)

    def CRZ(self, theta):
        return self.RZ(theta)

    def CU1(self, theta):
        return self.U1(theta)

    def CU2(self, phi, lam):
        return self.U2(phi, lam)

    def CU3(self, theta, phi, lam):
        return self.U3(theta, phi, lam)

    def U1(self, theta):
        return np.asarray(np.exp(1j * theta), dtype=self.dtype)

    @property
    def CNOT(self):
        return self.X

    @property
    def TOFFOLI(self):
        return self.X

    @property
    def CZ(self):
        return self.Z

    @property
    def CCZ(self):
        return self.Z

    @property
    def CY(self):
        return self.Y

    @property
    def CH(self):
        return self.H

    @property
    def CSX(self):
        return self.SX

    @property
    def CSXDG(self):
        return self.SXDG

    def DEUTSCH(self, theta):
        return 1j * self.RX(2 * theta)

    def fSim(self, theta, phi):
        c, s = np.cos(theta) + 0j, -1j * np.sin(theta)
        return np.array([c, s, s, c, np.exp(-1j * phi)], dtype=self.dtype)

    def GeneralizedfSim(self, u, phi):
        u = np.asarray(u)
        return np.array([u[0, 0], u[0, 1], u[1, 0], u[1, 1], np.exp(-1j * phi)], dtype=self.dtype)
