"""Fusion strategies for one circuit and a measured choice between them.

The reference leaves fusion to qibo, whose ``Circuit.fuse(max_qubits)`` merges runs of
gates into ``FusedGate`` blocks of up to k qubits that qibojit applies as dense
2^k x 2^k matrices (``cpu.py:535-537``, ``gpu.py:929-930``, the multi-target kernels
of ``raw_kernels.py:478-518``).  The engine has two ways to run a circuit:

* ``("blocks", k)``: the circuit fused into dense blocks of at most k qubits
  (``fuse_blocks``), one HBM pass per block through ``sv_apply_multi_qubit``; complex64
  blocks of 5 and 6 qubits run on the tensor cores;
* ``("passes", tile_bits)``: the cache-blocked fused passes (``FusedProgram``), many
  gates per HBM pass on 2^tile_bits-amplitude tiles, pass kernels specialised to the
  circuit at run time.

``autotune`` times every candidate on the device (CUDA events on the current stream,
after one untimed run that also compiles) and returns the fastest with the full table.
"""
from __future__ import annotations

from typing import Dict, Iterable, List, Optional, Sequence, Tuple

from . import gates as G


def fuse_blocks(circuit, max_qubits: int):
    """Greedy light-cone fusion into ``FusedGate`` blocks of at most ``max_qubits``
    qubits.  Every qubit remembers its latest block; a gate joins the latest blocks of
    its qubits, merged into one, when each of them is still the latest block on all of
    its own qubits and the merged qubit set stays within ``max_qubits``; otherwise the
    gate opens a new block.  Merged blocks act on disjoint qubits, so concatenating
    their gate lists keeps the order on every qubit.  A block depends on the blocks
    that preceded it on any of its qubits; blocks are emitted in a topological order
    of those dependencies (a block that can still be merged into is a sink, so merging
    never creates a cycle)."""
    from .fusion import _expand

    if max_qubits < 1:
        raise ValueError("blocks need at least one qubit")
    blocks: List[dict] = []  # {"qubits": set, "gates": list, "deps": set, "alive": bool}
    latest: Dict[int, int] = {}
    for g in _expand(circuit.queue):
        gq = set(int(q) for q in g.qubits)
        ids = sorted({latest[q] for q in gq if q in latest})
        cand = set(gq)
        ok = True
        for i in ids:
            cand |= blocks[i]["qubits"]
            ok &= all(latest.get(q) == i for q in blocks[i]["qubits"])
        if ok and ids and len(cand) <= max_qubits:
            keep = blocks[ids[0]]
            for i in ids[1:]:
                keep["gates"].extend(blocks[i]["gates"])
                keep["qubits"] |= blocks[i]["qubits"]
                keep["deps"] |= blocks[i]["deps"]
                blocks[i]["alive"] = False
            keep["deps"] -= set(ids)
            keep["gates"].append(g)
            keep["qubits"] |= gq
            for q in keep["qubits"]:
                latest[q] = ids[0]
        else:
            blocks.append({"qubits": set(gq), "gates": [g], "deps": set(ids), "alive": True})
            for q in gq:
                latest[q] = len(blocks) - 1
    out = G.Circuit(circuit.nqubits)
    for i in _topological(blocks):
        b = blocks[i]
        fg = G.FusedGate(*sorted(b["qubits"]))
        for h in b["gates"]:
            fg.append(h)
        out.add(fg)
    return out


def _topological(blocks: List[dict]) -> List[int]:
    """Indices of the surviving blocks, every block after all blocks it depends on
    (Kahn's algorithm, smallest index first among the ready ones)."""
    import heapq

    alive = [i for i, b in enumerate(blocks) if b["alive"]]
    indeg = {i: len(blocks[i]["deps"]) for i in alive}
    users: Dict[int, List[int]] = {i: [] for i in alive}
    for i in alive:
        for d in blocks[i]["deps"]:
            users[d].append(i)
    ready = [i for i in alive if indeg[i] == 0]
    heapq.heapify(ready)
    order = []
    while ready:
        i = heapq.heappop(ready)
        order.append(i)
        for u in users[i]:
            indeg[u] -= 1
            if indeg[u] == 0:
                heapq.heappush(ready, u)
    if len(order) != len(alive):
        raise RuntimeError("block dependencies form a cycle")
    return order


class _BlockRunner:
    def __init__(self, backend, circuit, k):
        self.backend = backend
        self.fused = fuse_blocks(circuit, k)
        self.nblocks = len(self.fused.queue)

    def run(self, state):
        n = self.fused.nqubits
        for g in self.fused.queue:
            state = self.backend.apply_gate(g, state, n)
        return state


def prepare(backend, circuit, dtype: str, strategy: Tuple[str, int]):
    """A runner with ``.run(state)`` for one strategy (compiled/fused, not yet run)."""
    kind, arg = strategy
    if kind == "passes":
        return backend.compile(circuit, dtype, tile_bits=int(arg), specialize=True)
    if kind == "blocks":
        return _BlockRunner(backend, circuit, int(arg))
    raise ValueError(f"unknown strategy {strategy}")


def autotune(backend, circuit, dtype: str, candidates: Optional[Sequence[Tuple[str, int]]] = None, reps: int = 1,
             state=None) -> Tuple[Tuple[str, int], List[dict]]:
    """Times each candidate strategy on ``circuit`` (from |0...0> unless ``state`` is
    given, which is left unchanged) and returns (best strategy, table sorted by time).
    Each row holds the strategy, milliseconds per run, HBM passes per run and gates/s."""
    import torch

    n = circuit.nqubits
    if candidates is None:
        candidates = [("passes", t) for t in (12, 13, 14) if t <= n] + [("blocks", k) for k in range(2, 7)]
    ngates = len(circuit.queue)
    work = backend.zero_state(n, dtype=dtype) if state is None else state.clone()
    stream = torch.cuda.current_stream()
    rows = []
    for strat in candidates:
        runner = prepare(backend, circuit, dtype, strat)
        src = backend.zero_state(n, dtype=dtype) if state is None else state
        work.copy_(src)
        runner.run(work)  # untimed: first launches, operand uploads
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        elapsed = 0.0
        for _ in range(max(1, reps)):
            work.copy_(src)
            e0.record(stream)
            runner.run(work)
            e1.record(stream)
            torch.cuda.synchronize()
            elapsed += e0.elapsed_time(e1)
        ms = elapsed / max(1, reps)
        passes = runner.stats()["passes"] if strat[0] == "passes" else runner.nblocks
        rows.append({"strategy": f"{strat[0]}:{strat[1]}", "ms": ms, "hbm_passes": passes,
                     "gates_per_s": ngates / (ms / 1000.0)})
        del runner
    rows.sort(key=lambda r: r["ms"])
    kind, arg = rows[0]["strategy"].split(":")
    return (kind, int(arg)), rows
