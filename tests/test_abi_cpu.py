"""CPU-only checks of the boundary: the engine library loads, exports every entry
point the header declares, and reports errors without touching a GPU."""
import ctypes
import os
import re
import shutil

import numpy as np
import pytest

from qibojit_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qibojit_gb300.h")


def _declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sv_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("engine library not built and nvcc unavailable")
        from qibojit_gb300 import build

        build.build()
    return _lib.load()


def test_header_and_binding_agree():
    assert _declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in _declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.sv_version() >= 100
    assert isinstance(_lib.last_error(), str)


def test_no_device_maps_to_import_error(lib):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.sv_context_create(0, ctypes.byref(h))
    assert rc == _lib.SV_ERR_NO_DEVICE
    with pytest.raises(ImportError):
        _lib.check(rc, "sv_context_create")


def test_null_context_is_rejected(lib):
    rc = lib.sv_apply_one_qubit(None, None, 0, 4, 0, None, 0, None, 0)
    assert rc == _lib.SV_ERR_ARG
    assert "context" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(rc)


def test_null_handles_are_rejected_by_batch_and_adjoint_entry_points(lib):
    """The batch executor switch and the adjoint specialiser check their handles before
    touching a device."""
    assert lib.sv_batch_set_executor(None, None, 1) == _lib.SV_ERR_ARG
    assert lib.sv_adjoint_specialize(None, None) == _lib.SV_ERR_ARG
    assert lib.sv_batch_pass_bytes(None, None) == _lib.SV_ERR_ARG
    assert lib.sv_batch_arith(None, None) == _lib.SV_ERR_ARG
    assert lib.sv_program_arith_per_amplitude(None, None) == _lib.SV_ERR_ARG


@pytest.mark.parametrize("rc,exc", [(_lib.SV_ERR_ARG, ValueError), (_lib.SV_ERR_OOM, RuntimeError),
                                    (_lib.SV_ERR_UNSUPPORTED, NotImplementedError),
                                    (_lib.SV_ERR_TIMEOUT, TimeoutError), (_lib.SV_ERR_CUDA, RuntimeError)])
def test_status_to_exception(lib, rc, exc):
    with pytest.raises(exc):
        _lib.check(rc, "x")


def test_int32_array():
    a, n = _lib.int32_array([3, 1, 2])
    assert n == 3 and list(a) == [3, 1, 2]
    assert _lib.int32_array([]) == (None, 0)


def test_noalloc_grid_rule(tmp_path):
    """The launch-size rule of sv_collapse_state_noalloc (csrc/sv_noalloc_grid.h),
    compiled with the host compiler: a reduction fits the static array up to 4094
    partials (one per block, capped at 8 blocks per SM), so any GPU of up to 511 SMs
    is accepted and a 512-SM one would be rejected."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "grid.cpp"
    src.write_text(
        '#include <stdio.h>\n#include "sv_noalloc_grid.h"\n'
        "int main() {\n"
        "  const long long works[] = {1, 255, 256, 257, 1LL << 20, 1LL << 30, 1LL << 36};\n"
        "  const int sms[] = {1, 152, 511, 512, 1000};\n"
        "  for (int s : sms) for (long long w : works) {\n"
        "    unsigned g = sv::noalloc_grid(w, s, 256);\n"
        "    printf(\"%d %lld %u %d\\n\", s, w, g, (int)sv::noalloc_norm_fits(g));\n"
        "  }\n  return 0;\n}\n")
    exe = tmp_path / "grid"
    import subprocess

    subprocess.run([cxx, "-std=c++17", "-I", os.path.join(ROOT, "qibojit_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        s, w, g, fits = (int(v) for v in line.split())
        want = max(1, min((w + 255) // 256, 8 * s))
        assert g == want
        assert fits == (g + 2 <= 4096)
        if s <= 511:
            assert fits
    assert any(line.split()[3] == "0" for line in out if line and line.split()[0] == "512")


def test_persistent_queue_order(tmp_path):
    """The persistent batch executor's queue (csrc/sv_persist_queue.h), compiled with the
    host compiler, on random group shapes: tickets are contiguous, counters disjoint,
    every group's passes appear in order with each pass waiting on its predecessor's
    counters, all of whose tickets precede it (so a single worker taking tickets in
    order never waits on unfinished work: the property the kernel's bounded waits rely
    on), and a circuit's tickets of one pass cover exactly its 2^tshift tiles."""
    import random
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "queue.cpp"
    src.write_text(
        '#include <stdio.h>\n#include "sv_persist_queue.h"\n'
        "int main() {\n"
        "  int ng;\n"
        "  while (scanf(\"%d\", &ng) == 1) {\n"
        "    std::vector<sv::PersistGroup> g(ng);\n"
        "    for (auto& x : g) scanf(\"%d %d %d\", &x.npasses, &x.ncirc, &x.tshift);\n"
        "    int nc = 0;\n"
        "    auto q = sv::persist_queue(g, &nc);\n"
        "    printf(\"%d %zu\\n\", nc, q.size());\n"
        "    for (auto& e : q) printf(\"%d %d %lld %lld %d %d %d %d\\n\", e.group, e.pass, (long long)e.first,\n"
        "                            (long long)e.ntickets, e.tshift, e.cshift, e.cnt, e.prev);\n"
        "  }\n  return 0;\n}\n")
    exe = tmp_path / "queue"
    subprocess.run([cxx, "-std=c++17", "-I", os.path.join(ROOT, "qibojit_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True)
    rng = random.Random(3)
    cases = [[(3, 2, 0)], [(1, 5, 4), (4, 3, 1), (2, 7, 9)]]
    for _ in range(40):
        cases.append([(rng.randint(1, 12), rng.randint(1, 300), rng.randint(0, 10)) for _ in range(rng.randint(1, 30))])
    text = "".join(f"{len(c)} " + " ".join(f"{p} {n} {t}" for p, n, t in c) + "\n" for c in cases)
    lines = subprocess.run([str(exe)], input=text, check=True, capture_output=True, text=True).stdout.split("\n")
    pos = 0
    for case in cases:
        ncounters, nentries = (int(v) for v in lines[pos].split())
        entries = [tuple(int(v) for v in lines[pos + 1 + i].split()) for i in range(nentries)]
        pos += 1 + nentries
        assert nentries == sum(p for p, _, _ in case)
        nxt, used, seen = 0, set(), {}
        for group, pss, first, nt, tshift, cshift, cnt, prev in entries:
            npasses, ncirc, gt = case[group]
            assert first == nxt and nt == ncirc << (tshift - cshift)
            assert tshift == gt and cshift == min(tshift, 2)
            assert (nt // ncirc) << cshift == 1 << tshift  # a circuit's tiles of this pass
            nxt = first + nt
            span = set(range(cnt, cnt + ncirc))
            assert not (span & used)
            used |= span
            if pss == 0:
                assert prev == -1
            else:
                before = seen[(group, pss - 1)]
                assert prev == before[0] and before[1] <= first  # predecessor entirely earlier
            seen[(group, pss)] = (cnt, first + nt)
        assert len(used) == ncounters
        for gi, (npasses, _, _) in enumerate(case):
            assert all((gi, r) in seen for r in range(npasses))
