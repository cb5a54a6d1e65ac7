"""Output of a running solver: VTK frames written without stalling the GPU.

The reference copies the whole state to the host synchronously every output interval and
hands it to a detached writer thread (src/sph/sph_run.cu:258-281, src/io/io.cu:154-279).
Here sph_snapshot_begin writes the original-order state into device buffers of the context and
copies it to pinned host buffers on a separate copy stream, so the steps launched next overlap
the copy.  Once a frame's copy has completed (the next frame() or close() waits for it on the
caller's thread), a writer thread writes its legacy-VTK file (sph_write_vtk).  Two host buffer
sets alternate, so one frame can be written while the next is copied.

    with FrameWriter(solver, "result") as fw:
        for i in range(frames):
            solver.step(out_every, stream=s)
            fw.frame(i * out_every, stream=s)
"""
from __future__ import annotations

import os
import queue
import threading

import numpy as np

from .api import call, ptr


def write_vtk(path: str, pos, vel, p, type_=None, binary: bool = True) -> None:
    """Legacy-VTK particle file from host arrays (the reference's output layout)."""
    pos = np.ascontiguousarray(pos, np.float32)
    vel = np.ascontiguousarray(vel, np.float32)
    p = np.ascontiguousarray(p, np.float32)
    t = None if type_ is None else np.ascontiguousarray(type_, np.int32)
    call("sph_write_vtk", os.fsencode(path), len(p), ptr(pos), ptr(vel), ptr(p), ptr(t),
         1 if binary else 0)


def read_vtk(path: str) -> dict:
    """Read back a file written by write_vtk (binary or text)."""
    with open(path, "rb") as f:
        data = f.read()
    lines = data.split(b"\n", 5)
    binary = lines[2].strip() == b"BINARY"
    n = int(lines[4].split()[1])
    out = {}
    if binary:
        off = data.index(b"POINTS")
        off = data.index(b"\n", off) + 1
        out["pos"] = np.frombuffer(data, ">f4", 3 * n, off).reshape(n, 3).astype(np.float32)
        off += 12 * n
        off = data.index(b"LOOKUP_TABLE DEFAULT\n", off) + len(b"LOOKUP_TABLE DEFAULT\n")
        out["p"] = np.frombuffer(data, ">f4", n, off).astype(np.float32)
        off += 4 * n
        off = data.index(b"VECTORS velocity float\n", off) + len(b"VECTORS velocity float\n")
        out["vel"] = np.frombuffer(data, ">f4", 3 * n, off).reshape(n, 3).astype(np.float32)
        off += 12 * n
        k = data.find(b"SCALARS type int 1\nLOOKUP_TABLE DEFAULT\n", off)
        if k >= 0:
            k += len(b"SCALARS type int 1\nLOOKUP_TABLE DEFAULT\n")
            out["type"] = np.frombuffer(data, ">i4", n, k).astype(np.int32)
        return out
    toks = data.split()
    i = toks.index(b"POINTS") + 3
    out["pos"] = np.array(toks[i:i + 3 * n], np.float32).reshape(n, 3)
    i = toks.index(b"DEFAULT", i) + 1
    out["p"] = np.array(toks[i:i + n], np.float32)
    i = toks.index(b"velocity", i) + 2
    out["vel"] = np.array(toks[i:i + 3 * n], np.float32).reshape(n, 3)
    if b"type" in toks[i + 3 * n:]:
        i = toks.index(b"DEFAULT", i + 3 * n) + 1
        out["type"] = np.array(toks[i:i + n], np.int32)
    return out


class _HostSet:
    """Pinned host buffers for one frame."""

    def __init__(self, n: int):
        import torch
        self.t = {"pos": torch.empty((n, 3), dtype=torch.float32).pin_memory(),
                  "vel": torch.empty((n, 3), dtype=torch.float32).pin_memory(),
                  "p": torch.empty(n, dtype=torch.float32).pin_memory(),
                  "type": torch.empty(n, dtype=torch.int32).pin_memory()}
        self.a = {k: v.numpy() for k, v in self.t.items()}
        self.done = threading.Event()
        self.done.set()


class FrameWriter:
    """Writes `<directory>/fluid_t=<step>.vtk` frames of a Solver asynchronously.  All calls on
    the solver stay on the caller's thread; the writer thread only writes files."""

    def __init__(self, sol, directory: str, binary: bool = True):
        os.makedirs(directory, exist_ok=True)
        self.sol, self.dir, self.binary = sol, directory, binary
        self.sets = [_HostSet(sol.n), _HostSet(sol.n)]
        self.next = 0
        self.inflight = None  # (step, host set) whose copies may still be running
        self.q: queue.Queue = queue.Queue()
        self.err: list = []
        self.written: list = []
        self.th = threading.Thread(target=self._run, daemon=True)
        self.th.start()

    def frame(self, step: int, stream=None) -> None:
        """Snapshot the current state (asynchronously) and queue the previous frame's file."""
        from .solver import _stream
        hs = self.sets[self.next]
        self.next ^= 1
        hs.done.wait()  # the frame written from this set two frames ago is on disk
        hs.done.clear()
        a = hs.a
        # begins only after the previous snapshot's copies have completed
        call("sph_snapshot_begin", self.sol.handle, ptr(a["pos"]), ptr(a["vel"]), None,
             ptr(a["p"]), ptr(a["type"]), _stream(stream))
        if self.inflight is not None:
            self.q.put(self.inflight)
        self.inflight = (step, hs)

    def _run(self) -> None:
        while True:
            item = self.q.get()
            if item is None:
                return
            step, hs = item
            try:
                path = os.path.join(self.dir, f"fluid_t={step}.vtk")
                write_vtk(path, hs.a["pos"], hs.a["vel"], hs.a["p"], hs.a["type"], self.binary)
                self.written.append(path)
            except Exception as e:  # reported by close()
                self.err.append(e)
            finally:
                hs.done.set()

    def close(self) -> list:
        """Wait for every frame to be copied and written; returns the files written."""
        if self.inflight is not None:
            call("sph_snapshot_wait", self.sol.handle)
            self.q.put(self.inflight)
            self.inflight = None
        self.q.put(None)
        self.th.join()
        if self.err:
            raise self.err[0]
        return self.written

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
