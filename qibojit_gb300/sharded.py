"""A state vector split over 2^g ranks by global qubits (one GPU per rank).

The reference runs a circuit on several GPUs by splitting the state into 2^g pieces
indexed by the g global qubits (``CupyBackend.execute_distributed_circuit``,
``src/qibojit/backends/gpu.py:646-739``): gates on local qubits run piece by piece,
and a gate on a global qubit first swaps that global qubit with a local one by
exchanging half-pieces between the two pieces that differ in it (``MultiGpuOps.swap``,
``gpu.py:1497-1507`` -> ``swap_pieces``, ``custom_operators/ops.py:127-137``); the
full state is reassembled with ``transpose_state`` (``ops.py:111-124``).  The
reference keeps the pieces in host memory and moves each through a device in turn.

Here each rank owns one piece in its own device memory for the whole run:

* Physical qubit p of the full 2^n index (bit n-p-1) is global for p < g (the rank
  index holds those g bits) and local otherwise (local qubit p-g of the piece).  A
  permutation maps the circuit's logical qubits onto physical ones; it starts as the
  identity and changes with every swap.
* A gate whose targets are all local runs on every piece through the rank's local
  executor (the engine's per-gate kernels on its GPU); controls on global qubits turn
  into a predicate on the rank index (ranks whose bits are not all 1 skip the gate).
* A gate with a global target first swaps that global qubit with the most significant
  free local qubit.  The exchanged halves are then the two contiguous halves of the
  pieces: rank r (global bit 0) sends its upper half to its partner r ^ bit and
  receives the partner's lower half in its place, one point-to-point exchange of
  2^(n-g-1) amplitudes per rank over torch.distributed (NCCL between GPUs; gloo for
  CPU ranks).  No collective is involved.

``gather`` reassembles the full state in logical qubit order on every rank (for
checks and small states).
"""
from __future__ import annotations

import copy
from typing import Callable, List, Optional

import numpy as np


class ShardedState:
    """One rank's piece of an n-qubit state split over all ranks of ``group``.

    ``apply_local(piece, nlocal, gate)`` applies ``gate`` (whose qubits are already
    local piece qubits) to the 1-D tensor ``piece`` in place and returns it; the
    default is the GB300 backend's ``apply_gate``."""

    def __init__(self, nqubits: int, piece, apply_local: Callable, group=None):
        import torch.distributed as dist

        self.dist = dist
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        g = self.world.bit_length() - 1
        if 1 << g != self.world:
            raise ValueError(f"the number of ranks must be a power of two, not {self.world}")
        if nqubits - g < 2:
            raise ValueError(f"{nqubits} qubits over {self.world} ranks leave fewer than 2 local qubits")
        self.nqubits, self.nglobal, self.nlocal = nqubits, g, nqubits - g
        if piece.numel() != 1 << self.nlocal:
            raise ValueError(f"a piece holds 2^{self.nlocal} amplitudes")
        self.piece = piece
        self.apply_local = apply_local
        self.phys = list(range(nqubits))  # logical qubit -> physical qubit
        self.swaps = 0

    # ----------------------------------------------------------------- creation
    @classmethod
    def zero_state(cls, nqubits: int, apply_local: Callable, dtype="complex128", device="cpu", group=None):
        import torch
        import torch.distributed as dist

        world = dist.get_world_size(group)
        nlocal = nqubits - (world.bit_length() - 1)
        tdt = {"complex128": torch.complex128, "complex64": torch.complex64}[str(dtype)]
        piece = torch.zeros(1 << nlocal, dtype=tdt, device=device)
        if dist.get_rank(group) == 0:
            piece[0] = 1
        return cls(nqubits, piece, apply_local, group)

    @classmethod
    def from_full(cls, state, apply_local: Callable, group=None):
        """Piece `rank` of a full state (every rank passes the same full tensor)."""
        import torch.distributed as dist

        world = dist.get_world_size(group)
        n = int(state.numel()).bit_length() - 1
        nlocal = n - (world.bit_length() - 1)
        r = dist.get_rank(group)
        piece = state.reshape(-1)[r << nlocal:(r + 1) << nlocal].clone()
        return cls(n, piece, apply_local, group)

    # ------------------------------------------------------------------ gates
    def _global_bit(self, p: int) -> int:
        """Rank-index bit of global physical qubit p (rank = top g bits of the index)."""
        return (self.rank >> (self.nglobal - p - 1)) & 1

    def swap_global(self, p_global: int, p_local: int) -> None:
        """Exchanges global physical qubit ``p_global`` with the most significant local
        physical qubit ``p_local`` (= nglobal): the pieces differing in the global bit
        trade halves, then the two physical qubits trade their logical owners."""
        import torch

        if p_local != self.nglobal:
            raise ValueError("swaps go through the most significant local qubit")
        bit = 1 << (self.nglobal - p_global - 1)
        partner = self.rank ^ bit
        half = 1 << (self.nlocal - 1)
        mine = self._global_bit(p_global)
        # global bit 0 keeps its lower half and trades its upper half for the
        # partner's lower half (swap_pieces, ops.py:127-137)
        send = self.piece[half:] if mine == 0 else self.piece[:half]
        # gloo moves host tensors only: device pieces are staged through host memory
        staged = send.is_cuda and self.dist.get_backend(self.group) == "gloo"
        out = send.cpu() if staged else send
        recv = torch.empty_like(out)
        ops = [self.dist.P2POp(self.dist.isend, out, partner, self.group),
               self.dist.P2POp(self.dist.irecv, recv, partner, self.group)]
        for req in self.dist.batch_isend_irecv(ops):
            req.wait()
        send.copy_(recv)
        a = self.phys.index(p_global)
        b = self.phys.index(p_local)
        self.phys[a], self.phys[b] = p_local, p_global
        self.swaps += 1

    def apply_gate(self, gate) -> None:
        targets = [int(t) for t in gate.target_qubits]
        controls = [int(c) for c in gate.control_qubits]
        used = set(self.phys[q] for q in targets + controls)
        for t in targets:
            if self.phys[t] < self.nglobal:
                # the most significant local qubit must be free: move its logical owner
                # elsewhere if this gate uses it
                if self.nglobal in used:
                    free = [p for p in range(self.nglobal + 1, self.nqubits) if p not in used]
                    if not free:
                        raise ValueError("no free local qubit for a global-local swap")
                    self._local_permute(self.nglobal, free[0])
                    used = set(self.phys[q] for q in targets + controls)
                self.swap_global(self.phys[t], self.nglobal)
                used = set(self.phys[q] for q in targets + controls)
        gctl = [self.phys[c] for c in controls if self.phys[c] < self.nglobal]
        if any(self._global_bit(p) == 0 for p in gctl):
            return  # a global control is 0 on this piece: the gate is the identity here
        local = copy.copy(gate)
        local.target_qubits = tuple(self.phys[t] - self.nglobal for t in targets)
        local.control_qubits = tuple(self.phys[c] - self.nglobal for c in controls if self.phys[c] >= self.nglobal)
        self.piece = self.apply_local(self.piece, self.nlocal, local)

    def _local_permute(self, pa: int, pb: int) -> None:
        """Swaps two local physical qubits inside every piece (a local SWAP gate on the
        data, then the two physical qubits trade their logical owners)."""
        from .gates import SWAP

        self.piece = self.apply_local(self.piece, self.nlocal, SWAP(pa - self.nglobal, pb - self.nglobal))
        a, b = self.phys.index(pa), self.phys.index(pb)
        self.phys[a], self.phys[b] = pb, pa

    def run(self, circuit) -> "ShardedState":
        if circuit.nqubits != self.nqubits:
            raise ValueError(f"a {circuit.nqubits}-qubit circuit on a {self.nqubits}-qubit state")
        for gate in circuit.queue:
            if type(gate).__name__ == "FusedGate":
                for g in gate.gates:
                    self.apply_gate(g)
            elif getattr(gate, "name", "") == "fanout":
                from .gates import CNOT

                for t in gate.target_qubits:
                    self.apply_gate(CNOT(gate.control_qubits[0], t))
            else:
                self.apply_gate(gate)
        return self

    # ----------------------------------------------------------------- gather
    def gather(self):
        """The full state in logical qubit order, on every rank."""
        import torch

        mine = self.piece
        if mine.is_cuda and self.dist.get_backend(self.group) == "gloo":
            mine = mine.cpu()
        pieces = [torch.empty_like(mine) for _ in range(self.world)]
        self.dist.all_gather(pieces, mine.contiguous(), group=self.group)
        full = torch.cat(pieces).reshape((2,) * self.nqubits)
        # axis p of `full` is physical qubit p; logical qubit q sits on axis phys[q]
        return full.permute(self.phys).reshape(-1).contiguous()


def gb300_local_executor(backend) -> Callable:
    """The rank's local executor on its GPU: the backend's per-gate kernels."""

    def apply(piece, nlocal, gate):
        return backend.apply_gate(gate, piece, nlocal)

    return apply
