"""Serving loop for heat solve requests (elfel_server).

Each request is the reference's heat problem (Elfel.jl
test/test_heat.jl:89-111) on a T3/T6 block mesh of a rectangle, with its own
conductivity, source and Dirichlet polynomial.  The library admits requests
as batch slots and device memory free up, keeps meshes, patterns and solver
structures resident for later requests with the same mesh, assembles each
admission wave in batched launches and iterates all running requests in the
same graph launches (continuous batching).
"""
import ctypes

import numpy as np

from . import _native as N

_METHODS = {"pcg64": N.ELFEL_PCG64, "pcg32_ir": N.ELFEL_PCG32_IR}


def heat_request(etype, nx, ny=None, kappa=1.0, Q=-6.0, dirichlet=(1.0, 0.0, 0.0, 1.0, 0.0, 2.0), lx=1.0, ly=1.0,
                 orientation="a", t_arrival=-1.0, keep_solution=False):
    """An elfel_heat_request; the default Dirichlet data is T = 1 + x^2 + 2 y^2
    (the exact solution of test/test_heat.jl:25 for Q = -6, kappa = 1)."""
    r = N.HeatRequest()
    r.nodes_per_elem = 3 if etype == "T3" else 6
    r.orientation = {"a": 0, "alternate": 1}[orientation]
    r.nx = int(nx)
    r.ny = int(nx if ny is None else ny)
    r.lx, r.ly = float(lx), float(ly)
    r.kappa, r.Q = float(kappa), float(Q)
    for i, v in enumerate(dirichlet):
        r.dirichlet[i] = float(v)
    r.t_arrival = float(t_arrival)
    r.keep_solution = int(bool(keep_solution))
    return r


class HeatServer:
    """elfel_server: admission by device memory, resident systems, continuous batching."""

    def __init__(self, method="pcg32_ir", batched=True, max_active=64, graphs_per_step=1, rtol=1e-10,
                 maxit=200000, keep_idle=True, mem_budget=0, ctx=None):
        self.ctx = ctx or N.default_context()
        self.lib = self.ctx.lib
        cfg = N.ServerConfig(_METHODS[method], int(bool(batched)), int(max_active), int(graphs_per_step),
                             float(rtol), int(maxit), int(bool(keep_idle)), int(mem_budget))
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.elfel_server_create(self.ctx.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self._holds_systems = True
        self._ndofs = {}
        self.ctx.adopt(self)

    def clock(self):
        t = ctypes.c_double()
        self.ctx.check(self.lib.elfel_server_clock(self.h, ctypes.byref(t)))
        return t.value

    def submit(self, req):
        i = ctypes.c_int64()
        self.ctx.check(self.lib.elfel_server_submit(self.h, ctypes.byref(req), ctypes.byref(i)))
        return i.value

    def step(self):
        """One loop step; returns (active, queued)."""
        a, q = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.lib.elfel_server_step(self.h, ctypes.byref(a), ctypes.byref(q)))
        return a.value, q.value

    def poll(self, cap=4096):
        """Completed requests since the last poll, as dicts."""
        buf = (N.ServeResult * cap)()
        n = ctypes.c_int32()
        self.ctx.check(self.lib.elfel_server_poll(self.h, buf, cap, ctypes.byref(n)))
        out = [buf[i].as_dict() for i in range(n.value)]
        for r in out:
            self._ndofs[r["id"]] = r["ndofs"]
        return out

    def solution(self, rid):
        T = np.empty(self._ndofs[rid])
        self.ctx.check(self.lib.elfel_server_solution(self.h, int(rid), N.ptr(T), T.shape[0]))
        return T

    def stats(self):
        s = N.ServerStats()
        self.ctx.check(self.lib.elfel_server_stats_read(self.h, ctypes.byref(s)))
        return s.as_dict()

    def drain(self):
        """Step until nothing is queued or running; returns the completed results."""
        out = []
        while True:
            a, q = self.step()
            out.extend(self.poll())
            if a == 0 and q == 0:
                out.extend(self.poll())
                return out

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.lib.elfel_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
