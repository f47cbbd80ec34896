"""Batched solves: many device-resident systems iterated together.

The reference solves one system at a time (``K[1:nu,1:nu] \\ (F - K*T)[1:nu]``,
Elfel.jl test/test_heat.jl:73-76).  ``BatchSolver`` admits any number of
assembled systems (``SysmatAssemblerGPU`` or a finished
``SysmatAssemblerSparse``) with the arguments of ``solve``; the library then
iterates all of them in the same launches, as captured CUDA graphs, and
systems may join while others are running.  Each system's arithmetic does not
depend on the rest of the batch: its solution is bit-identical alone and in a
mix.
"""
import ctypes

import numpy as np

from . import _native as N

_METHODS = {"pcg64": N.ELFEL_PCG64, "pcg32_ir": N.ELFEL_PCG32_IR}


def _handle_of(K):
    from .assemblers import SysmatAssemblerGPU, SysmatAssemblerSparse

    if isinstance(K, SysmatAssemblerGPU):
        return K._hd
    if isinstance(K, SysmatAssemblerSparse):
        if K._hd is None:
            raise ValueError("finish the assembler before solving")
        return K._hd
    raise TypeError("K must be a SysmatAssemblerGPU or a finished SysmatAssemblerSparse")


class BatchSolver:
    """elfel_batch: slots of systems solved together on one device."""

    _holds_systems = True

    def __init__(self, method="pcg32_ir", capacity=64, ctx=None):
        self.ctx = ctx or N.default_context()
        self.lib = self.ctx.lib
        if method not in _METHODS:
            raise ValueError(f"batched methods: {sorted(_METHODS)}")
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.elfel_batch_create(self.ctx.h, _METHODS[method], int(capacity), ctypes.byref(h)))
        self.h = h
        self.capacity = capacity
        self._slots = {}  # slot -> (handle, nrow, T array)
        self.ctx.adopt(self)

    def add(self, K, T, nu, F=None, rtol=1e-10, maxit=200000):
        """Admit solve!(T, K, F, nu); returns the slot.  T is not modified
        (the solution comes back from ``result``)."""
        hd = _handle_of(K)
        T = N.f64(T)
        Fa = N.f64(F) if F is not None else None
        slot = ctypes.c_int32()
        self.ctx.check(self.lib.elfel_batch_add(self.h, hd.h, N.ptr(Fa), N.ptr(T), int(nu), float(rtol), int(maxit),
                                                ctypes.byref(slot)))
        self._slots[slot.value] = (hd, T.shape[0])
        return slot.value

    def step(self, graphs=1):
        """Run graph launches over every active system; returns how many are still iterating."""
        a = ctypes.c_int32()
        self.ctx.check(self.lib.elfel_batch_step(self.h, int(graphs), ctypes.byref(a)))
        return a.value

    def done(self):
        """Slots whose solve finished and whose result was not taken."""
        n = ctypes.c_int32()
        buf = (ctypes.c_int32 * max(self.capacity, 1))()
        self.ctx.check(self.lib.elfel_batch_done(self.h, buf, self.capacity, ctypes.byref(n)))
        return [buf[i] for i in range(min(n.value, self.capacity))]

    def result(self, slot):
        """(T, stats) of a finished slot; frees the slot."""
        hd, nrow = self._slots[slot]
        T = np.empty(nrow)
        st = N.SolveStats()
        self.ctx.check(self.lib.elfel_batch_result(self.h, int(slot), N.ptr(T), ctypes.byref(st)))
        del self._slots[slot]
        return T, st.as_dict()

    def run(self, graphs=4):
        """Step until every admitted system has finished; {slot: (T, stats)}."""
        out = {}
        while True:
            active = self.step(graphs)
            for s in self.done():
                out[s] = self.result(s)
            if active == 0 and not self._slots:
                return out

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.lib.elfel_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
