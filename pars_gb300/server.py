"""Python handle on the continuous-batching request server (pars_server_*)."""
import ctypes

import numpy as np

from . import _lib
from ._lib import PARS_WANT_PAIRS, ParsError, lib


class Server:
    """Requests of any loaded plan are queued, admitted by free arena memory into a
    worker's launch (up to max_batch_docs per launch; 1 = the plain per-request
    path) and answered with host copies of their results (in a pool of pinned
    memory of result_mib MiB, 0 = 1024, while it has room)."""

    def __init__(self, device: int = 0, arena_bytes: int = 8 << 30, workers: int = 2,
                 max_batch_docs: int = 4096, result_mib: int = 0):
        cfg = _lib.ServerConfig(device, workers, arena_bytes, max_batch_docs, result_mib)
        h = ctypes.c_void_p()
        rc = lib().pars_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise ParsError(rc, "pars_server_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().pars_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_plan(self, plan: bytes) -> int:
        pid = ctypes.c_int(-1)
        buf = ctypes.create_string_buffer(plan, len(plan))
        rc = lib().pars_server_plan_load(self.handle, buf, len(plan), ctypes.byref(pid))
        if rc:
            raise ParsError(rc, "pars_server_plan_load")
        return pid.value

    def submit(self, plan_id: int, data_ptr: int, n: int, want_pairs: bool = False) -> int:
        """Queues a request; the host bytes at `data_ptr` must stay alive until done."""
        t = ctypes.c_uint64()
        rc = lib().pars_server_submit(self.handle, plan_id, ctypes.c_void_p(data_ptr), n,
                                      PARS_WANT_PAIRS if want_pairs else 0, ctypes.byref(t))
        if rc:
            raise ParsError(rc, "pars_server_submit")
        return t.value

    def done(self, ticket: int) -> bool:
        """Whether the request has finished (pars_server_poll; does not block)."""
        r = _lib.ServerResult()
        rc = lib().pars_server_poll(self.handle, ticket, ctypes.byref(r))
        if rc == _lib.PARS_EAGAIN:
            return False
        if rc:
            raise ParsError(rc, "pars_server_poll")
        return True

    def wait(self, ticket: int, release: bool = True, copy: bool = True) -> dict:
        """Blocks until the request is done; with copy=False only its record (no
        offsets or pairs) comes back."""
        r = _lib.ServerResult()
        rc = lib().pars_server_wait(self.handle, ticket, ctypes.byref(r))
        if rc:
            raise ParsError(rc, "pars_server_wait")
        n = int(r.n_struct)
        out = {
            "status": r.status, "n_struct": n, "batch_docs": r.batch_docs,
            "balanced": r.balanced, "well_formed": r.well_formed, "max_depth": r.max_depth,
            "unclosed_mode": r.unclosed_mode,
            "latency_ns": int(r.done_ns - r.submit_ns), "queue_ns": int(r.start_ns - r.submit_ns),
            "submit_ns": int(r.submit_ns), "done_ns": int(r.done_ns),
            "pos": np.ctypeslib.as_array(ctypes.cast(r.structural, ctypes.POINTER(ctypes.c_uint32)), (n,)).copy()
            if (n and copy) else (np.zeros(0, np.uint32) if copy else None),
            "pair": np.ctypeslib.as_array(ctypes.cast(r.pair_pos, ctypes.POINTER(ctypes.c_int32)), (n,)).copy()
            if (n and r.pair_pos and copy) else None,
        }
        if release:
            lib().pars_server_release(self.handle, ticket)
        return out
