"""Serving loop for many CG solves on different operators (afm_server_* in
include/afm.h): admission by HBM budget (lane-sized requests first), device-resident state, every
admitted request advanced by the server's progress thread, on its own stream or,
for small requests, in the serving lane (one launch for the FP32 iterations of
all of them)."""
import ctypes as C

import numpy as np

from ._native import AfmServerInfo, AfmSolveStats, check, libafm


class Server:
    def __init__(self, device=0, hbm_budget=0, max_active=0):
        self._lib = libafm()
        h = C.c_void_p()
        check(self._lib.afm_server_create(C.byref(h), int(device), int(hbm_budget), int(max_active)),
              "afm_server_create")
        self._h = h
        self._n = {}

    def submit(self, A, b, rtol=1e-8, inner_rtol=0.1):
        """Queues a solve of A x = b (A: aMatFree with maps and element matrices set; the server takes it
        over and A can no longer be used). Returns the request id."""
        bb = np.ascontiguousarray(b, dtype=np.float64)
        if len(bb) != A.n_dofs:
            raise ValueError("b has %d entries, the operator %d DoFs" % (len(bb), A.n_dofs))
        rid = C.c_uint64()
        check(self._lib.afm_server_submit(self._h, A._h, C.c_void_p(bb.ctypes.data), float(rtol), float(inner_rtol),
                                          C.byref(rid)), "afm_server_submit")
        A._h = None  # owned by the server now
        self._n[rid.value] = len(bb)
        return rid.value

    def set_lane(self, max_ke_bytes=8 << 20, iters_per_launch=32):
        """Requests whose FP32 element matrices take at most max_ke_bytes run their FP32 iterations in the
        serving lane (0: off), at most iters_per_launch iterations per launch."""
        check(self._lib.afm_server_set_lane(self._h, int(max_ke_bytes), int(iters_per_launch)),
              "afm_server_set_lane")

    def set_inner_format(self, fmt=4):
        """Symmetric inner format of the requests with 2^20 DoFs or more on their own streams (4: FP64 inner
        vectors on the corrected symmetric arena; 0 to 5 as aMatFree.set_symmetric_inner); smaller ones use 1."""
        check(self._lib.afm_server_set_inner_format(self._h, int(fmt)), "afm_server_set_inner_format")

    def set_priorities(self, enable=True):
        """Stream priority by request size (the lane and small requests first), or none."""
        check(self._lib.afm_server_set_priorities(self._h, int(bool(enable))), "afm_server_set_priorities")

    def info(self):
        """Counters of the serving lane: launches, requests carried, largest batch, requests per path."""
        i = AfmServerInfo()
        check(self._lib.afm_server_get_info(self._h, C.byref(i)), "afm_server_get_info")
        return {k: getattr(i, k) for k, _ in AfmServerInfo._fields_ if k != "reserved"}

    def poll(self):
        """One more round of progress without blocking; returns (queued, admitted)."""
        q, a = C.c_uint32(), C.c_uint32()
        check(self._lib.afm_server_poll(self._h, C.byref(q), C.byref(a)), "afm_server_poll")
        return q.value, a.value

    def take(self, rid):
        """(x, stats, times) of a finished request (times: submit, admit, start, done on the steady clock),
        or None while it runs. Raises AfmError if the solve failed."""
        x = np.empty(self._n[rid])
        st = AfmSolveStats()
        t = (C.c_double * 4)()
        fin = C.c_int()
        s = self._lib.afm_server_take(self._h, C.c_uint64(rid), C.byref(fin), C.c_void_p(x.ctypes.data),
                                      C.byref(st), t)
        if s == 0 and not fin.value:
            return None
        if fin.value:
            del self._n[rid]
        check(s, "afm_server_take")
        return x, st, tuple(t)

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.afm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
