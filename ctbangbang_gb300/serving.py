"""Python face of the request server (ctbb_server_*): continuous batching of
whole-scan reconstructions over library contexts.

    with Server(n_workers=3, device_budget_bytes=150 << 30) as srv:
        t = srv.submit(mr, h_scan, h_final)        # pinned host buffers
        res = srv.wait(t)                          # RequestResult
"""
import ctypes as C

from . import lib as L
from .structs import RequestResult


class Server:
    def __init__(self, n_workers, device_budget_bytes):
        self._lib = L.load()
        h = C.c_void_p()
        L.call("ctbb_server_create", int(n_workers), C.c_size_t(int(device_budget_bytes)), C.byref(h))
        self._h = h

    def submit(self, mr, h_scan, h_final, mu_water=0.0):
        """h_scan / h_final: ctypes float pointers (kept alive by the caller)."""
        t = C.c_uint64()
        L.call("ctbb_server_submit", self._h, C.byref(mr), h_scan, h_final, C.c_float(mu_water), C.byref(t))
        return t.value

    def wait(self, ticket):
        """The request's RequestResult; raises CtbbError if it failed."""
        res = RequestResult()
        L.call("ctbb_server_wait", self._h, C.c_uint64(ticket), C.byref(res))
        return res

    def close(self):
        if self._h:
            self._lib.ctbb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
