"""Static checks of the CUDA sources' stream use (no GPU needed).

Every device operation of the library runs on an explicit non-blocking
stream (a context's, a wave's or a solver's).  The legacy default stream is
not ordered with such streams, so a copy or memset issued there (cudaMemcpy,
cudaMemset without Async) can still be in flight when a kernel on the
solver's stream reads the data -- with index data (symmetric-vector maps,
solution segments, request lists) that is an out-of-range access.  A
device-wide synchronize stalls every other solver of the process.  Host
sources of asynchronous copies must outlive the copy: the request lists of
the serving waves are staged in pinned per-wave buffers.
"""

import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parents[1] / "madsdp.jl_gb300" / "csrc"


def _sources():
    files = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))
    assert files
    for f in files:
        # comments removed: only code counts
        text = re.sub(r"//[^\n]*", "", f.read_text())
        yield f.name, text


def test_no_legacy_stream_copies_or_memsets():
    bad = []
    for name, text in _sources():
        for call in ("cudaMemcpy(", "cudaMemset(", "cudaMemcpy2D(", "cudaDeviceSynchronize("):
            if call in text:
                bad.append(f"{name}: {call}")
    assert not bad, bad


def test_every_kernel_launch_names_a_stream():
    bad = []
    for name, text in _sources():
        for m in re.finditer(r"<<<(.*?)>>>", text, flags=re.S):
            args = [a for a in re.split(r",(?![^(]*\))", m.group(1))]
            if len(args) < 4:
                bad.append(f"{name}: <<<{m.group(1)}>>>")
    assert not bad, bad


def test_server_stages_wave_lists_in_pinned_memory():
    text = (CSRC / "server.cu").read_text()
    # the order list, init list and pending count go up from the wave's
    # pinned buffer, never from a vector or local that dies on return
    assert "cudaMemcpyAsync(w.dorder, horder" in text
    assert "cudaMemcpyAsync(w.dinit, hinit" in text
    assert "cudaMemcpyAsync(w.pending, hpend" in text
    assert "act.data()" not in text and "fresh.data()" not in text and "&cnt" not in text
