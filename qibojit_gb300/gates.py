"""Minimal gate and circuit objects with the attributes qibojit's backends read.

qibojit consumes qibo gates through a handful of attributes
(``src/qibojit/backends/cpu.py:433-450, 519-539, 565-569``): ``target_qubits``,
``control_qubits``, ``parameters``, ``name``, ``init_args`` and the class name,
which selects the kernel through ``GATE_OPS``.  When qibo is installed its gates
work with the GB300 backend unchanged; these classes provide the same surface so
the engine can be driven (and tested) without qibo.
"""
from __future__ import annotations

from typing import Iterable, List, Sequence

import numpy as np

from .matrices import Matrices


class Gate:
    name = "gate"
    ntargets = 1

    def __init__(self, *qubits, params: Sequence = ()):
        self.target_qubits = tuple(int(q) for q in qubits)
        self.control_qubits: tuple = ()
        self.parameters = tuple(params)
        self.init_args = list(qubits)
        self.init_kwargs = {}

    @property
    def qubits(self):
        return self.control_qubits + self.target_qubits

    def controlled_by(self, *q):
        self.control_qubits = tuple(int(x) for x in q)
        return self

    def base_matrix(self, dtype="complex128"):
        """Dense matrix acting on ``target_qubits`` only (controls not included)."""
        m = Matrices(dtype)
        name = _UNCONTROLLED.get(type(self).__name__, type(self).__name__)
        if name == "DEUTSCH":
            return 1j * m.RX(2 * self.parameters[0])
        attr = getattr(m, name)
        if callable(attr):
            return attr(*self.parameters) if self.parameters else attr(2 ** len(self.target_qubits))
        return attr

    def matrix(self, backend=None, dtype="complex128"):
        """Dense matrix on ``control_qubits + target_qubits`` (controls first)."""
        u = self.base_matrix(dtype)
        for _ in self.control_qubits:
            u = Matrices._controlled(u)
        return u

    def __repr__(self):
        return f"{type(self).__name__}(t={self.target_qubits}, c={self.control_qubits}, p={self.parameters})"


class ParametrizedGate(Gate):
    pass


# controlled gate class -> gate class of its target operation
_UNCONTROLLED = {"CNOT": "X", "CZ": "Z", "CY": "Y", "CH": "H", "CSX": "SX", "CSXDG": "SXDG",
                 "CRX": "RX", "CRY": "RY", "CRZ": "RZ", "CU1": "U1", "CU2": "U2", "CU3": "U3",
                 "TOFFOLI": "X", "CCZ": "Z", "FanOut": "X"}


def _fixed(cls_name, gname, ntargets=1, ncontrols=0):
    def __init__(self, *qubits):
        if len(qubits) != ntargets + ncontrols:
            raise ValueError(f"{cls_name} takes {ntargets + ncontrols} qubits")
        Gate.__init__(self, *qubits[ncontrols:])
        self.control_qubits = tuple(int(q) for q in qubits[:ncontrols])
        self.init_args = list(qubits)

    return type(cls_name, (Gate,), {"__init__": __init__, "name": gname, "ntargets": ntargets})


def _param(cls_name, gname, pnames, ntargets=1, ncontrols=0):
    def __init__(self, *args, **kwargs):
        nq = ntargets + ncontrols
        qubits, params = args[:nq], list(args[nq:])
        for p in pnames[len(params):]:
            params.append(kwargs[p])
        Gate.__init__(self, *qubits[ncontrols:], params=params)
        self.control_qubits = tuple(int(q) for q in qubits[:ncontrols])
        self.init_args = list(qubits)
        self.init_kwargs = dict(zip(pnames, params))

    return type(cls_name, (ParametrizedGate,), {"__init__": __init__, "name": gname, "ntargets": ntargets})


H = _fixed("H", "h")
X = _fixed("X", "x")
Y = _fixed("Y", "y")
Z = _fixed("Z", "z")
S = _fixed("S", "s")
SDG = _fixed("SDG", "sdg")
T = _fixed("T", "t")
TDG = _fixed("TDG", "tdg")
SX = _fixed("SX", "sx")
SXDG = _fixed("SXDG", "sxdg")
CNOT = _fixed("CNOT", "cx", 1, 1)
CZ = _fixed("CZ", "cz", 1, 1)
CY = _fixed("CY", "cy", 1, 1)
CH = _fixed("CH", "ch", 1, 1)
CSX = _fixed("CSX", "csx", 1, 1)
CSXDG = _fixed("CSXDG", "csxdg", 1, 1)
SWAP = _fixed("SWAP", "swap", 2)
TOFFOLI = _fixed("TOFFOLI", "ccx", 1, 2)
CCZ = _fixed("CCZ", "ccz", 1, 2)
RX = _param("RX", "rx", ["theta"])
RY = _param("RY", "ry", ["theta"])
RZ = _param("RZ", "rz", ["theta"])
U1 = _param("U1", "u1", ["theta"])
U2 = _param("U2", "u2", ["phi", "lam"])
U3 = _param("U3", "u3", ["theta", "phi", "lam"])
CRX = _param("CRX", "crx", ["theta"], 1, 1)
CRY = _param("CRY", "cry", ["theta"], 1, 1)
CRZ = _param("CRZ", "crz", ["theta"], 1, 1)
CU1 = _param("CU1", "cu1", ["theta"], 1, 1)
CU2 = _param("CU2", "cu2", ["phi", "lam"], 1, 1)
CU3 = _param("CU3", "cu3", ["theta", "phi", "lam"], 1, 1)
fSim = _param("fSim", "fsim", ["theta", "phi"], 2)
DEUTSCH = _param("DEUTSCH", "deutsch", ["theta"], 1, 2)


class GeneralizedfSim(ParametrizedGate):
    name = "generalizedfsim"

    def __init__(self, q0, q1, unitary, phi):
        super().__init__(q0, q1, params=(np.asarray(unitary), phi))


class Unitary(ParametrizedGate):
    name = "Unitary"

    def __init__(self, unitary, *qubits):
        super().__init__(*qubits, params=(np.asarray(unitary),))
        d = 2 ** len(qubits)
        if self.parameters[0].shape != (d, d):
            raise ValueError(f"Unitary on {len(qubits)} qubits needs a {d}x{d} matrix")


class FanOut(Gate):
    """CNOT from qubit q0 onto every other listed qubit."""

    name = "fanout"

    def __init__(self, *qubits):
        super().__init__(*qubits[1:])
        self.control_qubits = (int(qubits[0]),)
        self.init_args = list(qubits)


class FusedGate(Gate):
    """A run of gates merged into one dense matrix on the union of their qubits."""

    name = "fused"

    def __init__(self, *qubits):
        super().__init__(*sorted(qubits))
        self.gates: List[Gate] = []

    def append(self, gate: Gate):
        self.gates.append(gate)


class Channel:
    """A noise channel sum_k c_k U_k with the attributes NumbaBackend.apply_channel reads
    (cpu.py:400-415): ``coefficients``, one gate per coefficient in ``gates``,
    ``coefficient_sum`` and ``_all_unitary_operators``."""

    name = "channel"

    def __init__(self, coefficients: Sequence[float], gates: Sequence[Gate]):
        if len(coefficients) != len(gates):
            raise ValueError("a channel needs one coefficient per gate")
        self.coefficients = tuple(float(c) for c in coefficients)
        self.gates = tuple(gates)
        self.coefficient_sum = float(sum(self.coefficients))
        if not 0.0 <= self.coefficient_sum <= 1.0 + 1e-12 or min(self.coefficients, default=0.0) < 0.0:
            raise ValueError("channel coefficients must be probabilities summing to at most 1")
        self._all_unitary_operators = True

    @property
    def qubits(self):
        return tuple(sorted({q for g in self.gates for q in g.qubits}))

    @property
    def target_qubits(self):
        return self.qubits


class PauliNoiseChannel(Channel):
    """X, Y and Z on ``q`` with probabilities px, py, pz (zero ones are left out)."""

    name = "paulinoise"

    def __init__(self, q: int, px: float = 0.0, py: float = 0.0, pz: float = 0.0):
        pairs = [(p, cls(q)) for p, cls in ((px, X), (py, Y), (pz, Z)) if p > 0]
        super().__init__([p for p, _ in pairs], [g for _, g in pairs])


class UnitaryChannel(Channel):
    """Unitary matrices on given qubits with given probabilities: ``ops`` is a list of
    (qubits, matrix) pairs."""

    name = "unitarychannel"

    def __init__(self, probabilities: Sequence[float], ops: Sequence):
        super().__init__(probabilities, [Unitary(np.asarray(m), *qs) for qs, m in ops])


class Circuit:
    def __init__(self, nqubits: int):
        self.nqubits = int(nqubits)
        self.queue: List[Gate] = []

    def add(self, gate):
        if isinstance(gate, Iterable) and not isinstance(gate, Gate):
            for g in gate:
                self.add(g)
            return
        for q in gate.qubits:
            if not 0 <= q < self.nqubits:
                raise ValueError(f"gate {gate} acts outside a {self.nqubits}-qubit circuit")
        self.queue.append(gate)

    def __len__(self):
        return len(self.queue)

    def __call__(self, initial_state=None, backend=None):
        from . import get_backend

        return (backend or get_backend()).execute_circuit(self, initial_state)
