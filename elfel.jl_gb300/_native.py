"""ctypes binding of libelfel_gpu.so (the C ABI declared in include/elfel_gpu.h).

The library is built in-tree by ``nvcc_build.py``.  There is no CPU fallback: if
the library is missing, or no CUDA device is present when a context is
created, the calls raise.
"""
import ctypes
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libelfel_gpu.so")

ELFEL_OK = 0
ELFEL_ERR_ARG = 1
ELFEL_ERR_CUDA = 2
ELFEL_ERR_BUDGET = 3
ELFEL_ERR_NOT_CONVERGED = 4
ELFEL_ERR_STATE = 5
ELFEL_ERR_TIMEOUT = 6
ELFEL_ERR_UNSUPPORTED = 7

ELFEL_HEAT = 1
ELFEL_ELASTICITY = 2
ELFEL_STOKES = 3

ELFEL_SHAPE_TRIANGLE = 0
ELFEL_SHAPE_Q4 = 1
ELFEL_SHAPE_T4 = 2

ELFEL_PCG64 = 0
ELFEL_PCG32_IR = 1
ELFEL_MINRES64 = 2
ELFEL_MINRES32_IR = 3

_STATUS = {
    ELFEL_ERR_ARG: "invalid argument",
    ELFEL_ERR_CUDA: "CUDA error",
    ELFEL_ERR_BUDGET: "device memory budget exceeded",
    ELFEL_ERR_NOT_CONVERGED: "not converged",
    ELFEL_ERR_STATE: "call out of order",
    ELFEL_ERR_TIMEOUT: "device wait timed out",
    ELFEL_ERR_UNSUPPORTED: "unsupported",
}


class ElfelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_STATUS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class NotConverged(ElfelError):
    pass


_i64p = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class Space(ctypes.Structure):
    _fields_ = [("nodes_per_elem", ctypes.c_int32), ("ncomp", ctypes.c_int32), ("nel", ctypes.c_int64),
                ("nnodes", ctypes.c_int64), ("conn", _i64p), ("xy", _dp), ("eldofs", _i64p)]


class FusedDesc(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("npts", ctypes.c_int32), ("qp_coords", _dp), ("qp_weights", _dp),
                ("ndofs", ctypes.c_int64), ("u", Space), ("p", Space), ("shape", ctypes.c_int32),
                ("sdim", ctypes.c_int32)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("refinements", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("relres", ctypes.c_double), ("seconds", ctypes.c_double)]

    def as_dict(self):
        return {"iterations": self.iterations, "refinements": self.refinements, "converged": bool(self.converged),
                "relres": self.relres, "seconds": self.seconds}


class BlockDesc(ctypes.Structure):
    _fields_ = [("nodes_per_elem", ctypes.c_int32), ("orientation", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("npts", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("qp_coords", _dp), ("qp_weights", _dp)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("batched", ctypes.c_int32), ("max_active", ctypes.c_int32),
                ("graphs_per_step", ctypes.c_int32), ("rtol", ctypes.c_double), ("maxit", ctypes.c_int32),
                ("keep_idle", ctypes.c_int32), ("mem_budget", ctypes.c_int64)]


class HeatRequest(ctypes.Structure):
    _fields_ = [("nodes_per_elem", ctypes.c_int32), ("orientation", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("kappa", ctypes.c_double),
                ("Q", ctypes.c_double), ("dirichlet", ctypes.c_double * 6), ("t_arrival", ctypes.c_double),
                ("keep_solution", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class ServeResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("refinements", ctypes.c_int32), ("converged", ctypes.c_int32), ("relres", ctypes.c_double),
                ("t_arrival", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double),
                ("ndofs", ctypes.c_int64), ("nu", ctypes.c_int64), ("nel", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "completed", "rejected", "systems_created",
                                              "systems_reused", "systems_evicted", "resident_systems",
                                              "resident_bytes", "graph_launches", "solver_kernel_launches",
                                              "kernel_launches")] + \
        [(k, ctypes.c_double) for k in ("busy_seconds", "create_seconds", "assemble_seconds", "join_seconds",
                                        "iterate_seconds", "harvest_seconds")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes); the full exported surface of include/elfel_gpu.h
SIGNATURES = {
    "elfel_abi_version": (ctypes.c_int, []),
    "elfel_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(_vp)]),
    "elfel_ctx_destroy": (ctypes.c_int, [_vp]),
    "elfel_ctx_last_error": (ctypes.c_char_p, [_vp]),
    "elfel_ctx_memory": (ctypes.c_int, [_vp, _i64p, _i64p]),
    "elfel_ctx_set_stream": (ctypes.c_int, [_vp, _vp]),
    "elfel_ctx_stream": (_vp, [_vp]),
    "elfel_ctx_synchronize": (ctypes.c_int, [_vp]),
    "elfel_ctx_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
    "elfel_ctx_profile_read": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _dp, _i64p]),
    "elfel_sysmat_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "elfel_sysmat_destroy": (ctypes.c_int, [_vp]),
    "elfel_sysmat_start": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64]),
    "elfel_sysmat_assemble_coo": (ctypes.c_int, [_vp, _i64p, _i64p, _dp, ctypes.c_int64]),
    "elfel_sysmat_finish": (ctypes.c_int, [_vp, _i64p]),
    "elfel_sysmat_dims": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    "elfel_sysmat_csc": (ctypes.c_int, [_vp, _i64p, _i64p, _dp]),
    "elfel_sysmat_rhs": (ctypes.c_int, [_vp, _dp]),
    "elfel_sysvec_assemble": (ctypes.c_int, [_vp, ctypes.c_int64, _i64p, _dp, ctypes.c_int64, _dp]),
    "elfel_sysvec_assemble_noalloc": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp, ctypes.c_int64, _vp]),
    "elfel_fused_setup": (ctypes.c_int, [_vp, ctypes.POINTER(FusedDesc)]),
    "elfel_fused_set_geometry": (ctypes.c_int, [_vp, _dp]),
    "elfel_fused_heat": (ctypes.c_int, [_vp, _dp, ctypes.c_double]),
    "elfel_fused_elasticity": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _dp, _i64p,
                                              ctypes.c_int64, _dp]),
    "elfel_fused_stokes": (ctypes.c_int, [_vp, ctypes.c_double]),
    "elfel_solve": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                   ctypes.POINTER(SolveStats)]),
    "elfel_batch_create": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_vp)]),
    "elfel_batch_destroy": (ctypes.c_int, [_vp]),
    "elfel_batch_add": (ctypes.c_int, [_vp, _vp, _dp, _dp, ctypes.c_int64, ctypes.c_double, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_int32)]),
    "elfel_batch_step": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "elfel_batch_done": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32)]),
    "elfel_batch_result": (ctypes.c_int, [_vp, ctypes.c_int32, _dp, ctypes.POINTER(SolveStats)]),
    "elfel_ctx_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int32)]),
    "elfel_ctx_fma_rate": (ctypes.c_int, [_vp, ctypes.c_int32, _dp]),
    "elfel_error_l2": (ctypes.c_int, [_vp, _dp, ctypes.c_int32, _dp, ctypes.c_int32, _dp, _dp, _dp]),
    "elfel_fused_setup_block": (ctypes.c_int, [_vp, ctypes.POINTER(BlockDesc), _i64p, _i64p]),
    "elfel_block_dirichlet": (ctypes.c_int, [_vp, _dp, _dp]),
    "elfel_fused_tables": (ctypes.c_int, [_vp, _i64p, _dp, _i64p]),
    "elfel_fused_dims": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    "elfel_sysmat_tile_stats": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p, _i64p]),
    "elfel_fused_setup_numbered": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64p, _i64p, _i64p]),
    "elfel_number_dofs": (ctypes.c_int, [_vp, ctypes.c_int32, _i64p, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_i64p), _i64p]),
    "elfel_server_create": (ctypes.c_int, [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "elfel_server_destroy": (ctypes.c_int, [_vp]),
    "elfel_server_clock": (ctypes.c_int, [_vp, _dp]),
    "elfel_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(HeatRequest), _i64p]),
    "elfel_server_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "elfel_server_poll": (ctypes.c_int, [_vp, ctypes.POINTER(ServeResult), ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32)]),
    "elfel_server_solution": (ctypes.c_int, [_vp, ctypes.c_int64, _dp, ctypes.c_int64]),
    "elfel_server_stats_read": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
}

_LIB = None


def load(path=None):
    """Load the library (raises if it has not been built)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libelfel_gpu.so not built ({p}); run build() first. There is no CPU fallback.")
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = L
    return L


def ptr(a, t=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def i64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int64)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One device, one stream, a device-memory budget (elfel_ctx)."""

    def __init__(self, device=0, mem_budget=0):
        self.lib = load()
        h = _vp()
        rc = self.lib.elfel_ctx_create(int(device), int(mem_budget), ctypes.byref(h))
        if rc != ELFEL_OK:
            raise ElfelError(rc, f"cannot create a context on CUDA device {device}")
        self.h = h
        self.device = device
        self._children = weakref.WeakSet()  # handles to close before the context

    def adopt(self, child):
        self._children.add(child)

    def check(self, rc):
        if rc == ELFEL_OK:
            return
        msg = self.lib.elfel_ctx_last_error(self.h).decode(errors="replace")
        if rc == ELFEL_ERR_NOT_CONVERGED:
            raise NotConverged(rc, msg)
        raise ElfelError(rc, msg)

    def memory(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self.check(self.lib.elfel_ctx_memory(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_stream(self, stream_handle):
        self.check(self.lib.elfel_ctx_set_stream(self.h, _vp(stream_handle) if stream_handle else None))

    def stream(self):
        return self.lib.elfel_ctx_stream(self.h)

    def synchronize(self):
        self.check(self.lib.elfel_ctx_synchronize(self.h))

    def profile(self, enable=True):
        """Start (clearing earlier records) or stop recording per-phase CUDA events."""
        self.check(self.lib.elfel_ctx_profile(self.h, int(bool(enable))))

    def phases(self):
        """{phase name: (total device ms, launches)} recorded since profile(True)."""
        out = {}
        i = 0
        buf = ctypes.create_string_buffer(64)
        while True:
            ms, k = ctypes.c_double(), ctypes.c_int64()
            rc = self.lib.elfel_ctx_profile_read(self.h, i, buf, 64, ctypes.byref(ms), ctypes.byref(k))
            if rc == ELFEL_ERR_ARG:
                break
            self.check(rc)
            out[buf.value.decode()] = (ms.value, k.value)
            i += 1
        return out

    def fma_rate(self, bits=64):
        """Measured FMA throughput of the device, TFLOP/s (bits = 32 or 64)."""
        t = ctypes.c_double()
        self.check(self.lib.elfel_ctx_fma_rate(self.h, int(bits), ctypes.byref(t)))
        return t.value

    def tuning(self):
        """Autotuner records: [(line, chosen index)], one per tuned key."""
        out = []
        buf = ctypes.create_string_buffer(512)
        ch = ctypes.c_int32()
        i = 0
        while self.lib.elfel_ctx_tuning(self.h, i, buf, 512, ctypes.byref(ch)) == ELFEL_OK:
            out.append((buf.value.decode(), ch.value))
            i += 1
        return out

    def close(self):
        if getattr(self, "h", None):
            # batches hold systems: close them before the systems
            for ch in sorted(self._children, key=lambda o: 0 if getattr(o, "_holds_systems", False) else 1):
                ch.close()
            self.lib.elfel_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_DEFAULT = {}


def default_context(device=0):
    """A process-wide context per device, created on first use."""
    if device not in _DEFAULT:
        _DEFAULT[device] = Context(device)
    return _DEFAULT[device]
