"""Test infrastructure, not product code: ctypes wrapper of the CPU oracle
(oracle/_build/liboracle.so). Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import it.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

REF, SPEC = 0, 1
ART_SEED_MARKS, ART_FRONTIER0, ART_SUB_EDGES, ART_COMP_ROOT, ART_COMP_ID = 0, 1, 2, 3, 4
ART_INIT_LABELS, ART_FRONTIER_SIZES, ART_ROW_PTR, ART_COL_IND, ART_VALUES = 5, 6, 7, 8, 9
ART_LABELS, ART_STATUS = 10, 11
_FLOAT_ARTS = {ART_INIT_LABELS, ART_VALUES, ART_LABELS}


class BatchIn(ctypes.Structure):
    _fields_ = [
        ("inserted", ctypes.c_void_p), ("num_inserted", ctypes.c_int),
        ("gt_ids", ctypes.c_void_p), ("gt_labels", ctypes.c_void_p), ("num_gt", ctypes.c_int),
        ("deleted", ctypes.c_void_p), ("num_deleted", ctypes.c_int),
        ("edge_src", ctypes.c_void_p), ("edge_dst", ctypes.c_void_p), ("edge_weight", ctypes.c_void_p),
        ("num_edges", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("batch", ctypes.c_int), ("iterations", ctypes.c_int), ("num_components", ctypes.c_int),
        ("num_sub_edges", ctypes.c_int), ("hook_edges", ctypes.c_int), ("hook_truncated", ctypes.c_int),
        ("seed_frontier", ctypes.c_int), ("seed_marks", ctypes.c_int),
        ("affected_edges", ctypes.c_int64), ("frontier_visits", ctypes.c_int64),
        ("correct", ctypes.c_int64), ("total", ctypes.c_int64), ("accuracy", ctypes.c_float),
        ("init_branch", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_int, P, P, P, P, P, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_tau.restype = ctypes.c_float
        L.orc_tau.argtypes = [P]
        L.orc_apply_batch.restype = ctypes.c_int
        L.orc_apply_batch.argtypes = [P, ctypes.c_int, ctypes.POINTER(BatchIn), ctypes.POINTER(Stats)]
        L.orc_error.restype = ctypes.c_char_p
        L.orc_error.argtypes = [P]
        L.orc_labels.restype = P
        L.orc_labels.argtypes = [P]
        L.orc_artefact.restype = P
        L.orc_artefact.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
        L.orc_irlp.restype = ctypes.c_int
        L.orc_irlp.argtypes = [ctypes.c_int, P, P, P, P, P, P, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_int64)]
        _lib = L
    return _lib


def _p(a):
    return None if a is None or a.size == 0 else a.ctypes.data


class OracleRun:
    """The oracle's per-batch path over one graph."""

    def __init__(self, num_nodes, row_ptr, col_ind, values, true_labels=None, batch_map=None, *, tau=-1.0,
                 delta=1e-4, max_iterations=100000, semantics=REF, threads=1, record=False):
        self._arrays = [np.ascontiguousarray(row_ptr, np.int32), np.ascontiguousarray(col_ind, np.int32),
                        np.ascontiguousarray(values, np.float32),
                        None if true_labels is None else np.ascontiguousarray(true_labels, np.float32),
                        None if batch_map is None else np.ascontiguousarray(batch_map, np.int32)]
        a = self._arrays
        self.n = num_nodes
        self._h = lib().orc_create(num_nodes, a[0].ctypes.data, _p(a[1]), _p(a[2]), _p(a[3]), _p(a[4]), tau, delta,
                                   max_iterations, semantics, threads, int(bool(record)))
        if not self._h:
            raise ValueError("orc_create failed")

    @classmethod
    def from_problem(cls, p, **kw):
        return cls(p.num_nodes, p.row_ptr, p.col_ind, p.values, p.true_labels, p.batch_map(), **kw)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    @property
    def tau(self) -> float:
        return float(lib().orc_tau(self._h))

    def apply(self, b: int, batch) -> dict:
        keep = [np.ascontiguousarray(x) for x in (batch.inserted, batch.gt_ids, batch.gt_labels, batch.deleted,
                                                  batch.edge_src, batch.edge_dst, batch.edge_weight)]
        bi = BatchIn(_p(keep[0]), keep[0].size, _p(keep[1]), _p(keep[2]), keep[1].size, _p(keep[3]), keep[3].size,
                     _p(keep[4]), _p(keep[5]), _p(keep[6]), keep[4].size)
        st = Stats()
        if lib().orc_apply_batch(self._h, b, ctypes.byref(bi), ctypes.byref(st)) != 0:
            raise ValueError(lib().orc_error(self._h).decode())
        return st.as_dict()

    def labels(self) -> np.ndarray:
        p = lib().orc_labels(self._h)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)), (self.n,)).copy()

    def artefact(self, which: int) -> np.ndarray:
        cnt = ctypes.c_int64(0)
        p = lib().orc_artefact(self._h, which, ctypes.byref(cnt))
        t = ctypes.c_float if which in _FLOAT_ARTS else ctypes.c_int32
        if not p or cnt.value == 0:
            return np.zeros(0, dtype=np.float32 if which in _FLOAT_ARTS else np.int32)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(t)), (cnt.value,)).copy()


def irlp(num_nodes, row_ptr, col_ind, values, status, gt_class, labels, delta=1e-4, max_iterations=100000,
         threads=1):
    """IrLP on a snapshot; returns (labels, iterations, edge_visits)."""
    lab = np.ascontiguousarray(labels, np.float32).copy()
    arrs = [np.ascontiguousarray(x, t) for x, t in ((row_ptr, np.int32), (col_ind, np.int32), (values, np.float32),
                                                    (status, np.int32), (gt_class, np.int32))]
    vis = ctypes.c_int64(0)
    it = lib().orc_irlp(num_nodes, *[_p(a) if a.size else None for a in arrs], lab.ctypes.data, delta,
                        max_iterations, threads, ctypes.byref(vis))
    return lab, it, vis.value
