"""``GB300Backend``: qibojit's backend API on the GB300 engine.

The class mirrors the methods qibojit's ``NumbaBackend`` / ``CupyBackend`` expose
(``src/qibojit/backends/cpu.py:39-635``, ``src/qibojit/backends/gpu.py:44-1076``):
``apply_gate`` and the ``_one/_two/_multi_qubit_base`` kernels it dispatches to,
``apply_channel``, ``zero_state``, ``collapse_state``, ``calculate_probabilities``,
``sample_frequencies`` and ``measure_frequencies_op`` for state vectors and density
matrices, plus the dtype/device/seed/thread setters; ``execute_circuit`` runs fused
passes and ``execute_circuit_stream`` pipelines host states through them.  Every
amplitude operation is one call through the C ABI into the CUDA library; there is
no CPU path.  Device arrays are torch CUDA tensors (any contiguous CUDA tensor of
the backend's dtype works), used only as memory.
"""
from __future__ import annotations

import os
from collections import Counter
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _lib
from .matrices import CustomMatrices, Matrices

try:  # plug into qibo when it is installed
    from qibo.backends import Backend as _QiboBackend  # type: ignore
except Exception:  # pragma: no cover - qibo is optional
    _QiboBackend = object

# GATE_OPS, cpu.py:23-36
GATE_OPS = {
    "X": "apply_x",
    "CNOT": "apply_x",
    "TOFFOLI": "apply_x",
    "Y": "apply_y",
    "Z": "apply_z",
    "CY": "apply_y",
    "CZ": "apply_z",
    "U1": "apply_z_pow",
    "CU1": "apply_z_pow",
    "SWAP": "apply_swap",
    "fSim": "apply_fsim",
    "GeneralizedfSim": "apply_fsim",
}

# qibo's SHOT_METROPOLIS_THRESHOLD: below it qibo samples directly
SHOT_METROPOLIS_THRESHOLD = 100000

_TORCH_DTYPES = None


def _torch():
    import torch

    return torch


def _gpu_local_cpus(device: int):
    """CPUs next to the GPU (its PCI device's local_cpulist), or None if unknown."""
    torch = _torch()
    try:
        pr = torch.cuda.get_device_properties(device)
        busid = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{busid}/local_cpulist") as f:
            text = f.read().strip()
    except (OSError, AttributeError, RuntimeError):
        return None
    cpus = set()
    for part in text.split(","):
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus & os.sched_getaffinity(0) or None


def _torch_dtype(name: str):
    global _TORCH_DTYPES
    if _TORCH_DTYPES is None:
        t = _torch()
        _TORCH_DTYPES = {"complex128": t.complex128, "complex64": t.complex64,
                         "float64": t.float64, "float32": t.float32, "int64": t.int64,
                         "int32": t.int32}
    return _TORCH_DTYPES[name]


def _is_channel(gate) -> bool:
    """A qibo noise channel as NumbaBackend.apply_channel consumes it (cpu.py:400-415):
    coefficients with one gate each."""
    return hasattr(gate, "coefficients") and hasattr(gate, "gates")


def _inverse_target_matrix(gate, backend) -> np.ndarray:
    """U^-1 on a gate's targets, its controls kept: the target block (controls all 1,
    controls first) of the inverse of the gate's matrix.  The reference inverts the
    whole matrix (cpu.py:461-464), which is the same for uncontrolled gates."""
    full = np.linalg.inv(np.asarray(gate.matrix(backend), dtype=np.complex128))
    d = 1 << len(gate.target_qubits)
    return np.ascontiguousarray(full[-d:, -d:])


def _circuit_fingerprint(circuit) -> bytes:
    """Digest of a circuit's content: every gate's class, target and control qubits
    and parameter values (nested gates of a FusedGate included), in queue order."""
    import hashlib

    h = hashlib.blake2b(digest_size=16)

    def feed(gates):
        for g in gates:
            h.update(type(g).__name__.encode())
            h.update(repr((tuple(getattr(g, "target_qubits", ())), tuple(getattr(g, "control_qubits", ())))).encode())
            for p in getattr(g, "parameters", ()):
                h.update(np.ascontiguousarray(p, dtype=np.complex128).tobytes())
            coeffs = getattr(g, "coefficients", None)
            if coeffs is not None:
                h.update(np.asarray(coeffs, dtype=np.float64).tobytes())
            inner = getattr(g, "gates", None)
            if inner:
                h.update(b"[")
                feed(inner)
                h.update(b"]")

    feed(circuit.queue)
    return h.digest()


def _dtype_name(x) -> str:
    s = str(x)
    return s.replace("torch.", "").replace("numpy.", "").replace("<class '", "").replace("'>", "")


class GB300Backend(_QiboBackend):
    """State-vector backend running on one GB300 through the engine's C ABI."""

    def __init__(self, device: int = 0):
        if _QiboBackend is not object:
            super().__init__()
        torch = _torch()
        if not torch.cuda.is_available():
            raise ImportError("Could not detect a CUDA device for the gb300 platform.")
        self.name = "qibojit"
        self.platform = "gb300"
        self.device_index = int(device)
        self.device = f"/GPU:{device}"
        self._tdevice = torch.device("cuda", self.device_index)
        torch.cuda.set_device(self._tdevice)
        self.ctx = _lib.Context(self.device_index)
        self.lib = self.ctx.lib
        self.dtype = "complex128"
        self.matrices = Matrices(self.dtype)
        self.custom_matrices = CustomMatrices(self.dtype)
        try:
            self.nthreads = len(os.sched_getaffinity(0))
        except AttributeError:  # pragma: no cover
            self.nthreads = os.cpu_count() or 1
        self.versions = {"qibojit_gb300": "0.1.0", "engine": self.lib.sv_version()}
        self.tensor_types = (np.ndarray, torch.Tensor)
        self.supports_multigpu = False
        self.fusion = True
        # execute_circuit specialises a cached program's pass kernels (sv_program_specialize)
        # once it has run this many times; None keeps the interpreting tile kernel
        self.specialize_after: Optional[int] = 2
        self._programs = {}

    # ------------------------------------------------------------------ setters
    def set_dtype(self, dtype) -> None:
        dtype = _dtype_name(dtype)
        if dtype not in _lib.DTYPE_CODES:
            raise ValueError(f"Unsupported dtype {dtype}.")
        self.dtype = dtype
        self.matrices = Matrices(dtype)
        self.custom_matrices = CustomMatrices(dtype)

    def set_device(self, device: str) -> None:
        if "GPU" not in device:
            raise ValueError(f"Device {device} is not available for {self} backend.")
        idx = int(device.split(":")[-1]) if ":" in device else 0
        if idx != self.device_index:
            raise ValueError(f"Device {device} is not available for {self} backend (bound to GPU:{self.device_index}).")

    def set_threads(self, nthreads: int) -> None:
        """Number of Metropolis chains (the reference uses one chain per CPU thread)."""
        self.nthreads = int(nthreads)

    def set_seed(self, seed) -> None:
        if seed is not None:
            np.random.seed(seed)

    def __repr__(self):
        return "qibojit (gb300)"

    # ------------------------------------------------------------ array plumbing
    def cast(self, array, dtype=None, copy: bool = False):
        torch = _torch()
        dtype = _dtype_name(dtype) if dtype is not None else self.dtype
        tdt = _torch_dtype(dtype)
        if isinstance(array, torch.Tensor):
            out = array.to(device=self._tdevice, dtype=tdt)
            if copy and out.data_ptr() == array.data_ptr():
                out = out.clone()
            return out.contiguous()
        arr = np.asarray(array, dtype=dtype)
        return torch.from_numpy(np.ascontiguousarray(arr)).to(self._tdevice)

    def to_numpy(self, array):
        torch = _torch()
        if isinstance(array, torch.Tensor):
            return array.detach().cpu().numpy()
        return np.asarray(array)

    def _check_state(self, state, nqubits: Optional[int] = None) -> int:
        torch = _torch()
        if not isinstance(state, torch.Tensor) or not state.is_cuda:
            raise TypeError("GB300Backend operates on CUDA tensors; use backend.cast(state) first.")
        if not state.is_contiguous():
            raise ValueError("state must be contiguous")
        if nqubits is not None and state.numel() != (1 << int(nqubits)):
            raise ValueError(f"state has {state.numel()} amplitudes, not 2^{nqubits}")
        name = _dtype_name(state.dtype)
        if name not in _lib.DTYPE_CODES:
            raise TypeError(f"unsupported state dtype {name}")
        return _lib.DTYPE_CODES[name]

    def _operand(self, matrix, dtype: str):
        torch = _torch()
        if isinstance(matrix, torch.Tensor):
            matrix = matrix.detach().cpu().numpy()
        return np.ascontiguousarray(np.asarray(matrix, dtype=dtype).ravel())

    # -------------------------------------------------------------- state creation
    def host_buffer(self, nqubits: int, dtype=None):
        """A pinned host array of 2^nqubits amplitudes in memory next to the GPU.

        Host<->device copies of a state run at the link rate only from the GPU's local
        memory node; pinned pages are placed where the allocating thread runs, so the
        allocation runs on the GPU's local CPUs (the process affinity is restored)."""
        torch = _torch()
        tdt = _torch_dtype(_dtype_name(dtype) if dtype is not None else self.dtype)
        cpus = _gpu_local_cpus(self._tdevice.index or 0)
        old = os.sched_getaffinity(0)
        try:
            if cpus:
                os.sched_setaffinity(0, cpus)
            buf = torch.empty(1 << int(nqubits), dtype=tdt, pin_memory=True)
            buf.zero_()
        finally:
            if cpus:
                os.sched_setaffinity(0, old)
        return buf

    def zero_state(self, nqubits: int, density_matrix: bool = False, dtype=None):
        """|0...0> (or |0><0| as a 2^n x 2^n matrix, cpu.py:334-353)."""
        dtype = _dtype_name(dtype) if dtype is not None else self.dtype
        torch = _torch()
        nbits = 2 * nqubits if density_matrix else nqubits
        state = torch.empty(1 << nbits, dtype=_torch_dtype(dtype), device=self._tdevice)
        _lib.check(self.lib.sv_zero_state(self.ctx.handle, state.data_ptr(), _lib.DTYPE_CODES[dtype], int(nbits)),
                   "zero_state")
        return state.reshape(1 << nqubits, 1 << nqubits) if density_matrix else state

    # ------------------------------------------------------------- gate dispatch
    def apply_gate(self, gate, state, nqubits: int, inverse: bool = False):
        if len(tuple(state.shape)) == 2:
            return self._apply_gate_density_matrix(gate, state, nqubits, inverse)
        return self._apply_gate(gate, state, nqubits)

    def apply_channel(self, channel, state, nqubits: int):
        """A noise channel sum_k c_k U_k (cpu.py:359-367).  On a density matrix every
        branch is applied (cpu.py:400-415); on a state vector one branch is drawn from
        the coefficients (the rest of the probability keeps the state) with NumPy's
        global stream."""
        if len(tuple(state.shape)) == 2:
            return self._apply_channel_density_matrix(channel, state, nqubits)
        coeffs = [float(c) for c in channel.coefficients]
        probs = np.array(coeffs + [1.0 - sum(coeffs)], dtype=np.float64)
        index = int(np.random.choice(len(probs), p=probs))
        if index < len(channel.gates):
            state = self.apply_gate(channel.gates[index], state, nqubits)
        return state

    def _apply_channel_density_matrix(self, channel, state, nqubits: int):
        """new = (1 - sum c) rho + sum_k c_k U_k rho U_k^dagger (cpu.py:400-415), each
        branch on a copy of rho and accumulated by ``sv_axpby``.  The reference restores
        rho between branches by applying the inverse gate (unitary channels) or from a
        copy; here every branch starts from a copy, and the input is left unchanged."""
        torch = _torch()
        dt = self._check_state(state, 2 * int(nqubits))
        numel = state.numel()
        coeffs = [float(c) for c in channel.coefficients]
        total = float(getattr(channel, "coefficient_sum", sum(coeffs)))
        new = torch.empty_like(state)
        _lib.check(self.lib.sv_axpby(self.ctx.handle, dt, numel, state.data_ptr(), 1.0 - total, 0.0, new.data_ptr(),
                                     0.0, 0.0), "apply_channel")
        work = torch.empty_like(state)
        for coeff, gate in zip(coeffs, channel.gates):
            work.copy_(state)
            work = self._apply_gate_density_matrix(gate, work, nqubits)
            _lib.check(self.lib.sv_axpby(self.ctx.handle, dt, numel, work.data_ptr(), coeff, 0.0, new.data_ptr(),
                                         1.0, 0.0), "apply_channel")
        return new

    def _apply_gate_density_matrix(self, gate, state, nqubits: int, inverse: bool = False):
        """rho -> U rho U^dagger as two calls on the 2n-qubit vector (cpu.py:452-498): U
        on the row qubits (bits shifted up by n), conj(U) on the column qubits."""
        name = type(gate).__name__
        dtype = _dtype_name(state.dtype)
        if getattr(gate, "name", "") == "fanout":  # one CNOT per target, as on state vectors
            shape, n2, x = state.shape, 2 * nqubits, self.custom_matrices.X
            flat = state.reshape(-1)
            control = gate.control_qubits[0]
            for t in gate.target_qubits:
                q = np.array(sorted([nqubits - control - 1, nqubits - t - 1]), dtype=np.int32)
                flat = self._one_qubit_base(flat, n2, t, "apply_x", x, q + nqubits)
                flat = self._one_qubit_base(flat, n2, t + nqubits, "apply_x", x, q)
            return flat.reshape(shape)
        if inverse:
            matrix = _inverse_target_matrix(gate, self)
            gate = type("Inverse", (), {"target_qubits": tuple(gate.target_qubits),
                                         "control_qubits": tuple(gate.control_qubits),
                                         "parameters": (matrix,), "name": "inverse"})()
            name = "Unitary"
        else:
            matrix = self._as_custom_matrix(gate, dtype)
        qubits = self._create_qubits_tensor(gate, nqubits)
        qubits_dm = qubits + nqubits
        targets = gate.target_qubits
        targets_dm = tuple(q + nqubits for q in targets)
        shape = state.shape
        flat = state.reshape(-1)
        if not flat.is_contiguous():
            flat = flat.contiguous()
        n2 = 2 * nqubits
        if name in ("Y", "CY"):
            flat = self._one_qubit_base(flat, n2, *targets, "apply_y", matrix, qubits_dm)
            flat = self._one_qubit_base(flat, n2, *targets_dm, "apply_gate", np.conj(self.custom_matrices.Y),
                                        qubits)
        elif len(targets) == 1:
            op = GATE_OPS.get(name, "apply_gate")
            flat = self._one_qubit_base(flat, n2, *targets, op, matrix, qubits_dm)
            flat = self._one_qubit_base(flat, n2, *targets_dm, op, np.conj(matrix), qubits)
        elif len(targets) == 2:
            op = GATE_OPS.get(name, "apply_two_qubit_gate")
            flat = self._two_qubit_base(flat, n2, *targets, op, matrix, qubits_dm)
            flat = self._two_qubit_base(flat, n2, *targets_dm, op, np.conj(matrix), qubits)
        else:
            flat = self._multi_qubit_base(flat, n2, targets, matrix, qubits_dm)
            flat = self._multi_qubit_base(flat, n2, targets_dm, np.conj(matrix), qubits)
        return flat.reshape(shape)

    def _create_qubits_tensor(self, gate, nqubits: int):
        qubits = [nqubits - q - 1 for q in gate.control_qubits]
        qubits.extend(nqubits - q - 1 for q in gate.target_qubits)
        return np.array(sorted(qubits), dtype=np.int32)

    def _as_custom_matrix(self, gate, dtype: Optional[str] = None):
        """Kernel operand of a gate (cpu.py:519-539)."""
        dtype = dtype or self.dtype
        cm = self.custom_matrices if dtype == self.dtype else CustomMatrices(dtype)
        name = type(gate).__name__
        if name == "FusedGate":
            from .fusion import matrix_fused

            return matrix_fused(gate, dtype)
        if name == "Unitary":
            return self._operand(gate.parameters[0], dtype)
        _matrix = getattr(cm, name)
        if name == "FanOut":
            return cm.X
        if getattr(gate, "parameters", ()) and callable(_matrix):
            if name == "GeneralizedRBS":  # pragma: no cover
                raise NotImplementedError("GeneralizedRBS is not supported")
            return _matrix(*gate.parameters)
        return _matrix(2 ** len(gate.target_qubits)) if callable(_matrix) else _matrix

    def _apply_gate(self, gate, state, nqubits: int):
        dtype = _dtype_name(state.dtype)
        if getattr(gate, "name", "") == "fanout":
            return self._apply_fanout_gate(gate, state, nqubits)
        matrix = self._as_custom_matrix(gate, dtype)
        qubits = self._create_qubits_tensor(gate, nqubits)
        targets = gate.target_qubits
        if len(targets) == 1:
            op = GATE_OPS.get(type(gate).__name__, "apply_gate")
            return self._one_qubit_base(state, nqubits, *targets, op, matrix, qubits)
        if len(targets) == 2:
            op = GATE_OPS.get(type(gate).__name__, "apply_two_qubit_gate")
            return self._two_qubit_base(state, nqubits, *targets, op, matrix, qubits)
        return self._multi_qubit_base(state, nqubits, targets, matrix, qubits)

    def _apply_fanout_gate(self, gate, state, nqubits: int):
        control = gate.control_qubits[0]
        x = self.custom_matrices.X
        for target in gate.target_qubits:
            qubits = np.array(sorted([nqubits - control - 1, nqubits - target - 1]), dtype=np.int32)
            state = self._one_qubit_base(state, nqubits, target, "apply_x", x, qubits)
        return state

    def _one_qubit_base(self, state, nqubits: int, target: int, kernel: str, gate, qubits):
        dt = self._check_state(state, nqubits)
        op = self._operand(gate, _dtype_name(state.dtype)) if kernel in ("apply_gate", "apply_z_pow") else None
        q, nq = _lib.int32_array(qubits if qubits is not None else [])
        rc = self.lib.sv_apply_one_qubit(self.ctx.handle, state.data_ptr(), dt, int(nqubits),
                                         _lib.ONE_KINDS[kernel], None if op is None else op.ctypes.data,
                                         int(target), q, nq)
        _lib.check(rc, kernel)
        return state

    def _two_qubit_base(self, state, nqubits: int, target1: int, target2: int, kernel: str, gate, qubits):
        dt = self._check_state(state, nqubits)
        op = self._operand(gate, _dtype_name(state.dtype)) if kernel != "apply_swap" else None
        q, nq = _lib.int32_array(qubits if qubits is not None else [])
        rc = self.lib.sv_apply_two_qubit(self.ctx.handle, state.data_ptr(), dt, int(nqubits),
                                         _lib.TWO_KINDS[kernel], None if op is None else op.ctypes.data,
                                         int(target1), int(target2), q, nq)
        _lib.check(rc, kernel)
        return state

    def _multi_qubit_base(self, state, nqubits: int, targets, gate, qubits):
        dt = self._check_state(state, nqubits)
        op = self._operand(gate, _dtype_name(state.dtype))
        t, nt = _lib.int32_array(list(targets))
        if op.size != 1 << (2 * nt):
            raise ValueError(f"a gate on {nt} targets needs a {1 << nt}x{1 << nt} matrix")
        q, nq = _lib.int32_array(qubits if qubits is not None else [])
        rc = self.lib.sv_apply_multi_qubit(self.ctx.handle, state.data_ptr(), dt, int(nqubits), op.ctypes.data,
                                           t, nt, q, nq)
        _lib.check(rc, "apply_multi_qubit_gate")
        return state

    # ------------------------------------------------------------------ collapse
    def collapse_state(self, state, qubits: Sequence[int], shot, nqubits: int, normalize: bool = True,
                       density_matrix: bool = False):
        if hasattr(shot, "shape"):
            shot = int(np.asarray(self.to_numpy(shot)).ravel()[0])
        elif hasattr(shot, "__len__"):
            shot = int(shot[0])
        if density_matrix or len(tuple(state.shape)) == 2:
            return self._collapse_density_matrix(state, qubits, shot, nqubits, normalize)
        dt = self._check_state(state, nqubits)
        q, nq = _lib.int32_array(list(qubits))
        rc = self.lib.sv_collapse_state(self.ctx.handle, state.data_ptr(), dt, int(nqubits), q, nq, int(shot),
                                        int(bool(normalize)))
        _lib.check(rc, "collapse_state")
        return state

    def _collapse_density_matrix(self, rho, qubits: Sequence[int], shot: int, nqubits: int, normalize: bool):
        """rho -> P rho P (/ tr(P rho P)), P the projector of ``qubits`` onto the bits of
        ``shot`` (qubits[0] its most significant bit), in place.  On the 2n-qubit vector of
        rho this is the state-vector collapse of the row qubits and the column qubits
        (q + n) onto the shot twice over; the trace is the outcome's probability, taken
        from rho's diagonal before the projection."""
        n = int(nqubits)
        dt = self._check_state(rho, 2 * n)
        k = len(qubits)
        if not 0 <= shot < (1 << k):
            raise ValueError(f"shot {shot} is not an outcome of {k} qubits")
        if normalize:
            p = float(self.calculate_probabilities(rho, qubits, n, density_matrix=True,
                                                   out_dtype="float64")[shot].item())
        q, nq = _lib.int32_array(list(qubits) + [int(x) + n for x in qubits])
        rc = self.lib.sv_collapse_state(self.ctx.handle, rho.data_ptr(), dt, 2 * n, q, nq, (shot << k) | shot, 0)
        _lib.check(rc, "collapse_state")
        if normalize:
            with np.errstate(divide="ignore"):
                scale = float(np.float64(1.0) / np.float64(p))
            _lib.check(self.lib.sv_axpby(self.ctx.handle, dt, rho.numel(), rho.data_ptr(), scale, 0.0,
                                         rho.data_ptr(), 0.0, 0.0), "collapse_state")
        return rho

    # -------------------------------------------------------------- probabilities
    def calculate_probabilities(self, state, qubits: Sequence[int], nqubits: int, density_matrix: bool = False,
                                out_dtype: Optional[str] = None):
        """|psi|^2 marginalised on ``qubits``; float64 for complex128 states and float32
        for complex64 states (the state's real type, as qibo returns), summed in FP64."""
        if density_matrix:  # the real diagonal of rho, marginalised the same way
            dt = self._check_state(state, 2 * int(nqubits))
            entry = self.lib.sv_density_probabilities
        else:
            dt = self._check_state(state, nqubits)
            entry = self.lib.sv_probabilities
        if out_dtype is None:
            out_dtype = "float64" if dt in (_lib.SV_C128, _lib.SV_F64) else "float32"
        torch = _torch()
        out = torch.empty(1 << len(qubits), dtype=_torch_dtype(out_dtype), device=self._tdevice)
        q, nq = _lib.int32_array(list(qubits))
        rc = entry(self.ctx.handle, state.data_ptr(), dt, int(nqubits), q, nq, out.data_ptr(),
                   _lib.DTYPE_CODES[out_dtype])
        _lib.check(rc, "calculate_probabilities")
        return out

    # ------------------------------------------------------------------ sampling
    def measure_frequencies_op(self, frequencies, probs, nshots: int, nqubits: int, seed: int, nthreads: int):
        """ops.measure_frequencies (ops.py:82-108) on the GPU: same chains, same streams,
        same frequencies.  ``frequencies`` and ``probs`` may be numpy arrays (copied in and
        out) or CUDA tensors (updated in place)."""
        torch = _torch()
        host_out = None
        if not isinstance(frequencies, torch.Tensor):
            host_out = frequencies
            frequencies = torch.zeros(len(frequencies), dtype=torch.int64, device=self._tdevice)
            work = frequencies
        elif frequencies.dtype != torch.int64:
            work = torch.zeros(frequencies.shape[0], dtype=torch.int64, device=self._tdevice)
        else:
            work = frequencies
        probs = self.cast(probs, dtype=_dtype_name(probs.dtype))
        pdt = _lib.DTYPE_CODES[_dtype_name(probs.dtype)]
        if pdt not in (_lib.SV_F64, _lib.SV_F32):
            raise TypeError("probabilities must be float32 or float64")
        nstates = int(probs.shape[0])
        nbits = nstates.bit_length() - 1
        if nstates != 1 << nbits or work.shape[0] != nstates:
            raise ValueError("frequencies and probabilities need 2^n entries")
        rc = self.lib.sv_measure_frequencies(self.ctx.handle, work.data_ptr(), probs.data_ptr(), pdt, nbits,
                                             int(nshots), int(seed) & 0xFFFFFFFF, int(nthreads))
        _lib.check(rc, "measure_frequencies")
        if host_out is not None:
            host_out += work.cpu().numpy().astype(host_out.dtype)
            return host_out
        if work is not frequencies:
            frequencies += work.to(frequencies.dtype)
        return frequencies

    def _sampling_probs(self, probabilities):
        probs = self.cast(probabilities, dtype=_dtype_name(getattr(probabilities, "dtype", "float64")))
        if _dtype_name(probs.dtype) not in ("float64", "float32"):
            probs = probs.real.contiguous()
        nstates = int(probs.shape[0])
        nbits = nstates.bit_length() - 1
        if nstates != 1 << nbits:
            raise ValueError("probabilities need 2^n entries")
        return probs, _lib.DTYPE_CODES[_dtype_name(probs.dtype)], nbits

    def sample_shots(self, probabilities, nshots: int):
        """qibo's ``Backend.sample_shots``: ``numpy.random.choice(N, nshots, p=probabilities)``
        with the global NumPy stream (one ``random_sample`` draw per shot, as NumPy's
        choice takes them), each outcome searched on the device (``sv_sample_cdf``).
        Returns the outcomes as an int64 CUDA tensor."""
        torch = _torch()
        probs, pdt, nbits = self._sampling_probs(probabilities)
        uniforms = np.ascontiguousarray(np.random.random_sample(int(nshots)), dtype=np.float64)
        out = torch.empty(int(nshots), dtype=torch.int64, device=self._tdevice)
        _lib.check(self.lib.sv_sample_cdf(self.ctx.handle, probs.data_ptr(), pdt, nbits, uniforms.ctypes.data,
                                          int(nshots), None, out.data_ptr()), "sample_shots")
        return out

    def sample_frequencies(self, probabilities, nshots: int) -> Counter:
        """cpu.py:383-394: below SHOT_METROPOLIS_THRESHOLD shots, direct sampling (qibo's
        ``sample_shots`` path); from it on, the Metropolis chains of ``measure_frequencies``."""
        torch = _torch()
        probs, pdt, nbits = self._sampling_probs(probabilities)
        freqs = torch.zeros(probs.shape[0], dtype=torch.int64, device=self._tdevice)
        if nshots < SHOT_METROPOLIS_THRESHOLD:
            uniforms = np.ascontiguousarray(np.random.random_sample(int(nshots)), dtype=np.float64)
            _lib.check(self.lib.sv_sample_cdf(self.ctx.handle, probs.data_ptr(), pdt, nbits, uniforms.ctypes.data,
                                              int(nshots), freqs.data_ptr(), None), "sample_frequencies")
        else:
            seed = int(np.random.randint(0, int(1e8)))
            freqs = self.measure_frequencies_op(freqs, probs, nshots, 0, seed, self.nthreads)
        idx = torch.nonzero(freqs).flatten()
        return Counter(dict(zip(idx.cpu().tolist(), freqs[idx].cpu().tolist())))

    # ---------------------------------------------------------------- execution
    def compile(self, circuit, dtype: Optional[str] = None, tile_bits: int = 0, specialize: bool = False,
                density_matrix: bool = False):
        """Plans ``circuit`` into fused HBM passes (see ``qibojit_gb300.fusion``); with
        ``specialize`` also compiles pass kernels for its structure (seconds, once).  With
        ``density_matrix`` the program acts on the flattened 2^n x 2^n density matrix, a
        2n-qubit vector (each gate as U on the row qubits and conj(U) on the columns)."""
        from .fusion import FusedProgram, lower_density

        dtype = dtype or self.dtype
        nbits = 2 * circuit.nqubits if density_matrix else circuit.nqubits
        if specialize and not tile_bits:
            tile_bits = self._specialized_tile_bits(dtype, nbits)
        ops = lower_density(circuit.queue, circuit.nqubits) if density_matrix else None
        prog = FusedProgram(self.ctx, circuit.queue, nbits, dtype, tile_bits, ops=ops)
        return prog.specialize() if specialize else prog

    @staticmethod
    def _specialized_tile_bits(dtype: str, nqubits: int) -> int:
        """Specialised complex64 passes run fastest on the largest tiles (2^13 amplitudes,
        512 threads); complex128 keeps the planner's default."""
        return min(13, nqubits) if dtype == "complex64" else 0

    def execute_circuit(self, circuit, initial_state=None, nshots: Optional[int] = None,
                        fuse: Optional[bool] = None):
        """Runs ``circuit`` on ``initial_state`` (default |0...0>) and returns the state.

        With ``fuse`` (default: the backend's ``fusion`` flag) complex states of 8 or more
        qubits run as fused passes; otherwise gates are applied one by one (qibo's plain
        method, as the reference's ``execute_circuit`` does)."""
        n = circuit.nqubits
        if initial_state is None:
            state = self.zero_state(n)
        else:
            state = self.cast(initial_state, dtype=_dtype_name(getattr(initial_state, "dtype", self.dtype)),
                              copy=True)
        dtype = _dtype_name(state.dtype)
        fuse = self.fusion if fuse is None else fuse
        density = state.dim() == 2
        nbits = 2 * n if density else n
        channels = any(_is_channel(g) for g in circuit.queue)
        if fuse and nbits >= 8 and dtype in ("complex128", "complex64") and circuit.queue and not channels:
            # a density matrix runs as the 2n-qubit vector of rho: U on rows, conj(U) on columns
            flat = state.reshape(-1)
            self._cached_program(circuit, dtype, density_matrix=density).run(flat)
            return state
        for gate in circuit.queue:
            if _is_channel(gate):
                state = self.apply_channel(gate, state, n)
            else:
                state = self.apply_gate(gate, state, n)
        return state

    def _cached_program(self, circuit, dtype: str, upcoming_runs: int = 1, density_matrix: bool = False):
        """The program cache of execute_circuit (one entry), keyed by the circuit's
        content (every gate's class, qubits and parameter values), so a different or
        edited circuit never reuses a stale plan: a program that has run
        ``specialize_after`` times (counting the runs about to be made) is re-planned on
        the larger tile and its passes specialised (complex128 only in FP64 arithmetic)."""
        key = (_circuit_fingerprint(circuit), circuit.nqubits, dtype, bool(density_matrix))
        prog = self._programs.get(key)
        if prog is None:
            prog = self.compile(circuit, dtype, density_matrix=density_matrix)
            self._programs = {key: prog}
        # complex128 passes in double-word arithmetic run faster on the interpreting kernel
        # (compiled double-word passes stall on instruction fetch): they stay interpreted
        compiled_pays = dtype != "complex128" or getattr(self.ctx, "c128_arithmetic", "double-word") == "fp64"
        if (compiled_pays and not prog.specialized and self.specialize_after is not None
                and prog.runs + upcoming_runs - 1 >= self.specialize_after):
            runs = prog.runs
            prog = self.compile(circuit, dtype, specialize=True, density_matrix=density_matrix)
            prog.runs = runs
            self._programs = {key: prog}
        return prog

    def execute_circuit_stream(self, circuit, host_inputs, host_outputs):
        """Runs ``circuit`` on each pinned host state of ``host_inputs`` and writes each
        final state into the matching pinned tensor of ``host_outputs``.  With
        ``host_inputs=None`` every run starts from |0...0> prepared on the device (the
        reference's default initial state, ``cpu.py:334-353``) and only the final states
        cross the host link.

        States move through two device buffers on three CUDA streams: the upload of
        state k+1 and the read-back of state k-1 run while state k's passes do, so both
        directions of the host link and the GPU work at once.  Inputs may repeat (the
        same tensor for every k) and so may outputs (written in order, the last state
        wins); an output must not be a later step's input.  Returns when every state is
        back on the host."""
        torch = _torch()
        zero_start = host_inputs is None
        k_total = len(host_outputs) if zero_start else len(host_inputs)
        if len(host_outputs) != k_total:
            raise ValueError("need one output per input state")
        if k_total == 0:
            return host_outputs
        n = circuit.nqubits
        dtype = _dtype_name((host_outputs if zero_start else host_inputs)[0].dtype)
        if n < 8 or dtype not in ("complex128", "complex64") or not circuit.queue:
            for k, y in enumerate(host_outputs):
                y.copy_(self.execute_circuit(circuit, None if zero_start else host_inputs[k]))
            return host_outputs
        for t in ([] if zero_start else list(host_inputs)) + list(host_outputs):
            if t.is_cuda or t.numel() != (1 << n) or _dtype_name(t.dtype) != dtype:
                raise ValueError(f"host states must hold 2^{n} {dtype} amplitudes")
        prog = self._cached_program(circuit, dtype, k_total)
        tdt = _torch_dtype(dtype)
        dev = [torch.empty(1 << n, dtype=tdt, device=self._tdevice) for _ in range(min(2, k_total))]
        up, comp, down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        # The device buffers come from the caching allocator on the caller's current
        # stream, and earlier engine work sits on the context's own stream (the legacy
        # default stream, which does not order against non-blocking streams): finish the
        # latter and order the new streams after the former before touching anything.
        cur = torch.cuda.current_stream(self._tdevice)
        self.ctx.sync()
        up.wait_stream(cur)
        comp.wait_stream(cur)
        for buf in dev:
            for st in (up, comp, down):
                buf.record_stream(st)
        freed = [None] * len(dev)
        self.ctx.set_stream(comp.cuda_stream)
        try:
            dcode = _lib.DTYPE_CODES[dtype]
            for k in range(k_total):
                b = k % len(dev)
                if zero_start:
                    if freed[b] is not None:
                        comp.wait_event(freed[b])
                    _lib.check(self.lib.sv_zero_state(self.ctx.handle, dev[b].data_ptr(), dcode, n), "zero_state")
                else:
                    with torch.cuda.stream(up):
                        if freed[b] is not None:
                            up.wait_event(freed[b])
                        dev[b].copy_(host_inputs[k], non_blocking=True)
                        loaded = torch.cuda.Event()
                        loaded.record(up)
                    comp.wait_event(loaded)
                prog.run(dev[b])
                computed = torch.cuda.Event()
                computed.record(comp)
                with torch.cuda.stream(down):
                    down.wait_event(computed)
                    host_outputs[k].copy_(dev[b], non_blocking=True)
                    freed[b] = torch.cuda.Event()
                    freed[b].record(down)
        finally:
            for st in (up, comp, down):
                st.synchronize()
            cur.wait_stream(down)
            self.ctx.set_stream(0)
        return host_outputs

    # --------------------------------------------------------- FP64 reductions
    def inner_product(self, a, b, nqubits: int) -> complex:
        """<a|b> accumulated in FP64 (states may differ in precision)."""
        import ctypes

        da, db = self._check_state(a, nqubits), self._check_state(b, nqubits)
        out = (ctypes.c_double * 2)()
        _lib.check(self.lib.sv_inner_product(self.ctx.handle, a.data_ptr(), da, b.data_ptr(), db, int(nqubits), out),
                   "inner_product")
        return complex(out[0], out[1])

    def max_abs_diff(self, a, b, nqubits: int) -> float:
        import ctypes

        da, db = self._check_state(a, nqubits), self._check_state(b, nqubits)
        out = (ctypes.c_double * 1)()
        _lib.check(self.lib.sv_max_abs_diff(self.ctx.handle, a.data_ptr(), da, b.data_ptr(), db, int(nqubits), out),
                   "max_abs_diff")
        return out[0]

    def expectation_z(self, state, qubits: Sequence[int], nqubits: int) -> float:
        """<Z_{q1} Z_{q2} ...> in FP64; an empty list gives the squared norm."""
        import ctypes

        dt = self._check_state(state, nqubits)
        q, nq = _lib.int32_array(list(qubits))
        out = (ctypes.c_double * 1)()
        _lib.check(self.lib.sv_expectation_z(self.ctx.handle, state.data_ptr(), dt, int(nqubits), q, nq, out),
                   "expectation_z")
        return out[0]

    def norm2(self, state, nqubits: int) -> float:
        return self.expectation_z(state, [], nqubits)

    def assert_allclose(self, value, target, rtol=1e-7, atol=0.0):
        np.testing.assert_allclose(self.to_numpy(value), self.to_numpy(target), rtol=rtol, atol=atol)

    def synchronize(self) -> None:
        self.ctx.sync()
