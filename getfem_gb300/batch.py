"""Batched assembly of many independent meshes in a few launches.

A GetFEM user assembling many small problems calls ga_workspace::assembly
once per workspace; here the K + R assembly of every workspace of a batch
runs as one persistent element-pass launch per element type and one
row-gather launch per component count and valence class
(gfgpu_batch_assemble), which a CUDA graph can capture and replay
(coefficients changed in place between replays are picked up).

    b = Batch([ws1, ws2, ...])       # affine-simplex workspaces
    b.tune()                         # element-pass grid by measurement
    b.assemble()                     # every K and R, on the device
    g = b.graph(pre=perturb)         # torch.cuda.CUDAGraph of pre() + assemble
    g.replay()
"""
from __future__ import annotations

import ctypes as C

from . import _lib as L


def _stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Batch:
    def __init__(self, workspaces):
        lib = L.lib()
        self.workspaces = list(workspaces)
        self.plans = []
        for ws in self.workspaces:
            g = ws.groups[0]
            h = ws._plan(g, g.order1)
            ws._upload(h, g.order1, need_u=True)
            # the first order-2 assembly builds the plan's CSR pattern
            L.check(lib.gfgpu_assemble(h, 2, L.WITH_VECTOR, None))
            L.check(lib.gfgpu_sync(h))
            self.plans.append(h)
        arr = (C.c_void_p * len(self.plans))(*[h.value for h in self.plans])
        self.h = C.c_void_p()
        L.check(lib.gfgpu_batch_create(arr, len(self.plans), C.byref(self.h)))

    def elements(self) -> int:
        return L.lib().gfgpu_batch_elements(self.h)

    def assemble(self, stream=None):
        L.check(L.lib().gfgpu_batch_assemble(self.h, _stream_ptr(stream)))

    def sync(self, stream=None):
        L.check(L.lib().gfgpu_batch_sync(self.h, _stream_ptr(stream)))

    def tune(self, stream=None):
        """Element-pass grid (tuned) and the number of row-gather launches
        (one per component count and valence class)."""
        ge, gg = C.c_int32(), C.c_int32()
        L.check(L.lib().gfgpu_batch_tune(self.h, _stream_ptr(stream), C.byref(ge), C.byref(gg)))
        return ge.value, gg.value

    def graph(self, pre=None):
        """A torch.cuda.CUDAGraph replaying pre() followed by the batched
        assembly (pre: torch work on the capture stream, e.g. coefficients
        recomputed in place from a perturbation buffer)."""
        import torch
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):
                if pre is not None:
                    pre()
                self.assemble(s)
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            if pre is not None:
                pre()
            self.assemble(torch.cuda.current_stream())
        return g

    def matrix(self, i):
        return self.workspaces[i]._collect_matrix([self.plans[i]],
                                                  self.workspaces[i].groups[0].var.mf.nb_dof())

    def vector(self, i):
        return self.workspaces[i]._collect_vector([self.plans[i]],
                                                  self.workspaces[i].groups[0].var.mf.nb_dof())

    def __del__(self):
        try:
            if L._lib is not None and self.h:
                L.lib().gfgpu_batch_destroy(self.h)
                self.h = C.c_void_p()
        except Exception:
            pass
