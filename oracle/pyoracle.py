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
        L.orc_set_fp64.restype = ctypes.c_int
        L.orc_set_fp64.argtypes = [P, ctypes.c_int]
        L.orc_labels64.restype = P
        L.orc_labels64.argtypes = [P]
        L.orc_shadow_iterations.restype = ctypes.c_int
        L.orc_shadow_iterations.argtypes = [P]
        L.orc_generate.restype = P
        L.orc_generate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_float,
                                   ctypes.c_float]
        L.orc_problem_free.argtypes = [P]
        L.orc_problem_num_nodes.restype = ctypes.c_int
        L.orc_problem_num_nodes.argtypes = [P]
        L.orc_problem_num_edges.restype = ctypes.c_int64
        L.orc_problem_num_edges.argtypes = [P]
        for name in ("row_ptr", "col_ind", "values", "true_labels"):
            f = getattr(L, "orc_problem_" + name)
            f.restype = P
            f.argtypes = [P]
        L.orc_problem_num_batches.restype = ctypes.c_int
        L.orc_problem_num_batches.argtypes = [P]
        L.orc_problem_batch.restype = ctypes.c_int
        L.orc_problem_batch.argtypes = [P, ctypes.c_int, ctypes.POINTER(BatchIn)]
        L.orc_irlp.restype = ctypes.c_int
        L.orc_irlp.argtypes = [ctypes.c_int, P, P, P, P, P, P, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_int64)]
        _lib = L
    return _lib


def _p(a):
    return None if a is None or a.size == 0 else a.ctypes.data


class OracleBatch:
    """One batch's arrays (the fields of the product's Batch)."""

    FIELDS = ("inserted", "gt_ids", "gt_labels", "deleted", "edge_src", "edge_dst", "edge_weight")

    def __init__(self, **arrays):
        for k in self.FIELDS:
            setattr(self, k, arrays[k])


class OracleProblem:
    """The reference generator's output, made by the oracle's own restatement
    (generate_oracle.cpp): the same attributes as the product's Problem, with
    no product code loaded."""

    def __init__(self, num_nodes: int, avg_degree: int, num_batches: int, seed: int = 42,
                 gt_fraction: float = 0.01, deleted_fraction: float = 0.09):
        L = lib()
        h = L.orc_generate(num_nodes, avg_degree, num_batches, seed, gt_fraction, deleted_fraction)
        if not h:
            raise ValueError("orc_generate failed")
        try:
            def cp(p, cnt, t):
                if not cnt:
                    return np.zeros(0, dtype=np.dtype(t))
                return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(t)), (cnt,)).copy()
            self.num_nodes = L.orc_problem_num_nodes(h)
            n, m = self.num_nodes, L.orc_problem_num_edges(h)
            self.row_ptr = cp(L.orc_problem_row_ptr(h), n + 1, ctypes.c_int32)
            self.col_ind = cp(L.orc_problem_col_ind(h), m, ctypes.c_int32)
            self.values = cp(L.orc_problem_values(h), m, ctypes.c_float)
            self.true_labels = cp(L.orc_problem_true_labels(h), n, ctypes.c_float)
            self.batches = []
            for b in range(L.orc_problem_num_batches(h)):
                v = BatchIn()
                if L.orc_problem_batch(h, b, ctypes.byref(v)) != 0:
                    raise ValueError("orc_problem_batch failed")
                i32, f32 = ctypes.c_int32, ctypes.c_float
                self.batches.append(OracleBatch(
                    inserted=cp(v.inserted, v.num_inserted, i32), gt_ids=cp(v.gt_ids, v.num_gt, i32),
                    gt_labels=cp(v.gt_labels, v.num_gt, f32), deleted=cp(v.deleted, v.num_deleted, i32),
                    edge_src=cp(v.edge_src, v.num_edges, i32), edge_dst=cp(v.edge_dst, v.num_edges, i32),
                    edge_weight=cp(v.edge_weight, v.num_edges, f32)))
        finally:
            L.orc_problem_free(h)

    @property
    def num_edges(self) -> int:
        return int(self.col_ind.size)

    def batch_map(self) -> np.ndarray:
        """Batch of (last) arrival per vertex, -1 if never (src/dynLP.cu:193-198)."""
        m = np.full(self.num_nodes, -1, dtype=np.int32)
        for b, bt in enumerate(self.batches):
            m[bt.inserted] = b
        return m


class OracleRun:
    """The oracle's per-batch path over one graph. fp64=True (or 1): the same
    schedule in double precision; fp64=2: the fp32 run plus a double shadow of
    each batch's propagation from the same state (labels64(),
    shadow_iterations())."""

    def __init__(self, num_nodes, row_ptr, col_ind, values, true_labels=None, batch_map=None, *, tau=-1.0,
                 delta=1e-4, max_iterations=100000, semantics=REF, threads=1, record=False, fp64=False):
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
        if fp64:
            lib().orc_set_fp64(self._h, int(fp64))
        self.fp64 = int(fp64)

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

    def shadow_iterations(self) -> int:
        return int(lib().orc_shadow_iterations(self._h))

    def labels64(self) -> np.ndarray:
        p = lib().orc_labels64(self._h)
        if not p:
            raise ValueError("not an FP64 run")
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), (self.n,)).copy()

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


# --------------------------------------------------------------------------
# The reference's own kernels (oracle/_ref/ref_kernels, built on a GPU
# machine from the guarded copy of the reference's sources; see
# ref_kernels.cu). Test infrastructure like the rest of this module.

REF_KERNELS = HERE / "_ref" / "ref_kernels"
REF_SOURCES = HERE / "_ref" / "src" / ".guarded"


def build_ref_kernels() -> Path | None:
    """Builds oracle/_ref/ref_kernels from the guarded source copy when that
    copy is present; returns the binary, or None without the copy."""
    if not REF_SOURCES.exists():
        return None
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "refkern"], check=True)
    return REF_KERNELS


def run_ref_kernels(n: int, degree: int, batches: int, seed: int, max_iter: int, out: Path, record: bool,
                    timeout: float = 1800.0) -> dict:
    """Runs the reference's runDynLP on the GPU and reads what it recorded."""
    cmd = [str(REF_KERNELS), str(n), str(degree), str(batches), str(seed), str(max_iter), str(out)]
    if record:
        cmd.append("record")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, timeout=timeout)
    return read_ref_dump(out)


def read_ref_dump(path: Path) -> dict:
    buf = Path(path).read_bytes()
    if buf[:8] != b"DLPREFK1":
        raise ValueError("not a ref_kernels dump")
    off = 8

    def i64():
        nonlocal off
        v = int(np.frombuffer(buf, np.int64, 1, off)[0])
        off += 8
        return v

    def vec(dt):
        nonlocal off
        cnt = i64()
        a = np.frombuffer(buf, dt, cnt, off).copy()
        off += cnt * np.dtype(dt).itemsize
        return a

    n, nb, record = i64(), i64(), i64()
    tau = float(np.frombuffer(buf, np.float32, 1, off)[0])
    off += 4
    batches = []
    for _ in range(nb):
        head = np.frombuffer(buf, np.int32, 5, off)
        off += 20
        rec = {"num_new_edges": int(head[0]), "num_sub_edges": int(head[1]), "hook_edges": int(head[2]),
               "num_components": int(head[3]), "iterations": int(head[4]),
               "comp_id": vec(np.int32), "init_labels": vec(np.float32),
               "seed_marks": vec(np.int32), "labels": vec(np.float32)}
        # the propagation launcher's inputs (empty unless recorded)
        for name, dt in (("in_row_ptr", np.int32), ("in_col_ind", np.int32), ("in_values", np.float32),
                         ("in_labels", np.float32), ("in_status", np.int32), ("in_gt", np.int32),
                         ("in_affected", np.int32)):
            rec[name] = vec(dt)
        batches.append(rec)
    return {"n": n, "record": bool(record), "tau": tau, "batches": batches, "batch_ms": vec(np.float32),
            "accuracy": vec(np.float32), "final_labels": vec(np.float32)}
