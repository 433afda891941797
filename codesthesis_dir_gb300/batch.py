"""Batched Dirichlet Poisson solve (gb_batch_*): many independent
nabla^2 psi = f problems on n x n vertex grids (n = 2^m + 1) of uneven size.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _L


def offsets(sizes):
    sizes = np.asarray(sizes, dtype=np.int64)
    off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        off[1:] = np.cumsum(sizes ** 2)[:-1]
    return off, int(np.sum(sizes ** 2))


def autotune(sizes, precision, d_f, d_psi, nu1=2, nu2=2, tune_nu=False, rtol=1e-10, max_cycles=100, reps=3,
             cache_path=None):
    """gb_batch_autotune: times the candidate configurations of this size
    mix on the device with the right-hand side at device address d_f (d_psi:
    device scratch of the same size) and returns (winner, table of every
    candidate timed, from_cache), each a dict of gb_batch_tuning's fields."""
    L = _L.load()
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    best = _L.BatchTuning()
    table = (_L.BatchTuning * 512)()
    nt, hit = C.c_int(), C.c_int()
    _L.check(L.gb_batch_autotune(len(sizes), sizes.ctypes.data_as(C.POINTER(C.c_int)), precision, nu1, nu2,
                                 1 if tune_nu else 0, rtol, max_cycles, d_f, d_psi, reps,
                                 cache_path.encode() if cache_path else None, C.byref(best), table, 512,
                                 C.byref(nt), C.byref(hit)), "gb_batch_autotune")
    return best.as_dict(), [table[i].as_dict() for i in range(nt.value)], bool(hit.value)


class BatchPoisson:
    def __init__(self, sizes, precision=_L.BATCH_FP64, nu1=2, nu2=2, rtol=1e-10, max_cycles=100, inner=1,
                 exec_mode=None, tuning=None):
        """tuning: a dict of gb_batch_tuning's fields (e.g. autotune()'s
        winner); it replaces nu1, nu2, inner and exec_mode."""
        L = _L.load()
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.offsets, self.total = offsets(self.sizes)
        h = C.c_void_p()
        if tuning is not None:
            t = _L.BatchTuning(**{k: tuning[k] for k in ("nu1", "nu2", "inner", "local_n", "fuse", "exec")})
            _L.check(L.gb_batch_create_tuned(len(self.sizes), self.sizes.ctypes.data_as(C.POINTER(C.c_int)),
                                             precision, rtol, max_cycles, C.byref(t), C.byref(h)),
                     "gb_batch_create_tuned")
            inner, exec_mode = 1, None
        else:
            _L.check(L.gb_batch_create(len(self.sizes), self.sizes.ctypes.data_as(C.POINTER(C.c_int)), precision,
                                       nu1, nu2, rtol, max_cycles, C.byref(h)), "gb_batch_create")
        self._h = h
        self.nprob = len(self.sizes)
        if inner != 1:
            _L.check(L.gb_batch_set_inner_cycles(h, inner), "gb_batch_set_inner_cycles")
        if exec_mode is not None:
            _L.check(L.gb_batch_set_exec(h, exec_mode), "gb_batch_set_exec")

    def solve_device(self, d_f: int, d_psi: int, stream: int = 0):
        """d_f, d_psi: device addresses of packed float64 arrays."""
        cyc = np.zeros(self.nprob, dtype=np.int32)
        rr = np.zeros(self.nprob)
        st = _L.load().gb_batch_solve_device(self._h, d_f, d_psi, cyc.ctypes.data, rr.ctypes.data, stream or None)
        return st, cyc, rr

    def solve_host(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == self.total
        psi = np.zeros(self.total)
        cyc = np.zeros(self.nprob, dtype=np.int32)
        rr = np.zeros(self.nprob)
        st = _L.load().gb_batch_solve_host(self._h, f.ctypes.data, psi.ctypes.data, cyc.ctypes.data,
                                           rr.ctypes.data)
        return st, psi, cyc, rr

    def solve_stream(self, fs):
        """Solves a sequence of right-hand sides through the pipelined
        host-buffer calls (gb_batch_submit_host / gb_batch_drain): each
        upload and download overlaps a neighbouring call's solve.  Returns
        one (status, psi, cycles, relres) per right-hand side."""
        L = _L.load()
        keep, out, sts = [], [], []
        for f in fs:
            f = np.ascontiguousarray(f, dtype=np.float64)
            assert f.size == self.total
            psi = np.zeros(self.total)
            cyc = np.zeros(self.nprob, dtype=np.int32)
            rr = np.zeros(self.nprob)
            keep.append(f)
            out.append((psi, cyc, rr))
            sts.append(L.gb_batch_submit_host(self._h, f.ctypes.data, psi.ctypes.data, cyc.ctypes.data,
                                              rr.ctypes.data))
        sts.append(L.gb_batch_drain(self._h))
        # a submit returns the status of the solve submitted before it
        return [(sts[i + 1],) + out[i] for i in range(len(out))]

    def last_launches(self):
        return int(_L.load().gb_batch_last_launches(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _L.load().gb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
