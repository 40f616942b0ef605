"""Serving: resident form factors and rigid-transform scene queries.

The server (``pi_server_*`` in include/pointint_gb300.h) keeps each library
object's form factors resident on the device in its local frame.  A query
names library objects and gives each a rigid transform x' = R x + t on top of
its DoFs; translations become phases e^{i k . c} inside the tensor-core
contraction, and only rotated objects have their form factors evaluated.
Queries are admitted by a worker thread into batches that run as CUDA graphs
while later queries keep arriving (continuous batching).  No reference
counterpart: the reference recomputes every form factor on every call.

    srv = Server(kg, library_objects)
    t = srv.submit([0, 3, 3, 7], translations=T, rotations=R)
    V = srv.wait(t)                      # (4, 4) float64, 1/(8 pi^3) applied
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, ServerConfig, Query, ServerStats, CONTRACT_FP16X3, CONTRACT_BF16X3
from .geometry import SceneObject
from .kgrid import KGrid

PRECISIONS = {"fp16x3": CONTRACT_FP16X3, "bf16x3": CONTRACT_BF16X3}
STATE_NAMES = {0: "pending", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}


@dataclass
class Ticket:
    id: int
    n: int
    V: np.ndarray            # filled by the server before the ticket reads as done
    _keep: tuple             # host arrays the C side reads until the call returns


class Server:
    """A resident-J query server on the current CUDA device."""

    def __init__(self, kg: KGrid, library: list[SceneObject], *, hbm_budget_bytes: int = 0,
                 max_batch_queries: int = 0, max_batch_rows: int = 0, max_batch_evals: int = 0,
                 inflight_batches: int = 0, precision: str = "fp16x3", use_graphs: bool = True,
                 autotune: bool = True, items_per_sm: float = 0.0):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self._kg = kg                                   # keeps the device k-grid alive
        self._objs = [o.as_c() for o in library]
        self._hold = library
        arr = (_lib.PiObject * len(self._objs))(*self._objs)
        cfg = ServerConfig(hbm_budget_bytes, max_batch_queries, max_batch_rows, max_batch_evals, inflight_batches,
                           PRECISIONS[precision], 1 if use_graphs else 0, 1 if autotune else 0,
                           int(round(4 * items_per_sm)))
        h = ctypes.c_void_p()
        check(_lib.lib().pi_server_create(kg.handle(), arr, len(self._objs), ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.n_library = len(library)

    def submit(self, objects, rotations=None, translations=None) -> Ticket:
        obj = np.ascontiguousarray(objects, dtype=np.int32).reshape(-1)
        n = len(obj)
        R = None if rotations is None else np.ascontiguousarray(rotations, dtype=np.float64).reshape(n, 9)
        T = None if translations is None else np.ascontiguousarray(translations, dtype=np.float64).reshape(n, 3)
        V = np.empty((n, n), dtype=np.float64)
        q = Query(n, 0, obj.ctypes.data, None if R is None else R.ctypes.data, None if T is None else T.ctypes.data)
        tid = ctypes.c_uint64()
        check(_lib.lib().pi_server_submit(self._h, ctypes.byref(q), V.ctypes.data, ctypes.byref(tid)))
        return Ticket(int(tid.value), n, V, (obj, R, T))

    def poll(self, t: Ticket) -> str:
        st = ctypes.c_int32()
        check(_lib.lib().pi_server_poll(self._h, t.id, ctypes.byref(st)))
        return STATE_NAMES[st.value]

    def wait(self, t: Ticket, timeout: float | None = None) -> np.ndarray:
        check(_lib.lib().pi_server_wait(self._h, t.id, -1.0 if timeout is None else float(timeout)))
        return t.V

    def cancel(self, t: Ticket) -> None:
        check(_lib.lib().pi_server_cancel(self._h, t.id))

    def times(self, t: Ticket) -> tuple[int, int, int]:
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(_lib.lib().pi_server_times(self._h, t.id, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def release(self, t: Ticket) -> None:
        check(_lib.lib().pi_server_release(self._h, t.id))

    def stats(self) -> dict:
        st = ServerStats()
        check(_lib.lib().pi_server_stats_get(self._h, ctypes.byref(st)))
        out = {name: getattr(st, name) for name, _ in ServerStats._fields_
               if name not in ("tuned_items_per_sm", "tuned_k_splits")}
        out["tuned_items_per_sm"] = [v / 4 for v in st.tuned_items_per_sm]
        out["tuned_k_splits"] = list(st.tuned_k_splits)
        return out

    def query(self, objects, rotations=None, translations=None) -> np.ndarray:
        """Submit one scene and wait for its volume matrix."""
        t = self.submit(objects, rotations, translations)
        V = self.wait(t)
        self.release(t)
        return V

    def close(self) -> None:
        if getattr(self, "_h", None):
            check(_lib.lib().pi_server_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
