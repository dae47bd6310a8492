"""GB300-native DynLP per-batch update path (Python binding of the C ABI).

The compute lives in libdynlp_gb300.so (hand-written sm_103a CUDA); this
package wraps its C ABI for tests, benchmarks and Python callers:

    Problem   seeded synthetic graph + batches (the reference generator's output)
    Session   one dynamic graph resident on the GPU; apply() runs a whole batch
    DeviceArray  a device buffer for the step launchers and device-resident inputs
    launchers    the reference's five step launchers on device arrays
"""
from __future__ import annotations

import ctypes
import os
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _native as _n
from ._native import DlpError, SEMANTICS_REF, SEMANTICS_SPEC, ARITH_IEEE, ARITH_REFERENCE_FAST_MATH  # noqa: F401

__all__ = ["Problem", "Session", "DeviceArray", "IrlpSnapshot", "irlp_snapshot", "irlp", "DlpError",
           "SEMANTICS_REF", "SEMANTICS_SPEC", "device_count", "batch_map"]


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None or a.size == 0 else a.ctypes.data


def device_count() -> int:
    c = ctypes.c_int(0)
    _n.check(_n.lib().dlp_device_count(ctypes.byref(c)))
    return c.value


@dataclass
class Batch:
    inserted: np.ndarray
    gt_ids: np.ndarray
    gt_labels: np.ndarray
    deleted: np.ndarray
    edge_src: np.ndarray
    edge_dst: np.ndarray
    edge_weight: np.ndarray

    @staticmethod
    def make(inserted=(), gt_ids=(), gt_labels=(), deleted=(), edge_src=(), edge_dst=(), edge_weight=()):
        i32 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.int32).reshape(-1))
        f32 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1))
        return Batch(i32(inserted), i32(gt_ids), f32(gt_labels), i32(deleted), i32(edge_src), i32(edge_dst),
                     f32(edge_weight))

    def view(self) -> _n.BatchView:
        v = _n.BatchView()
        v.inserted, v.num_inserted = _ptr(self.inserted), self.inserted.size
        v.gt_ids, v.gt_labels, v.num_gt = _ptr(self.gt_ids), _ptr(self.gt_labels), self.gt_ids.size
        v.deleted, v.num_deleted = _ptr(self.deleted), self.deleted.size
        v.edge_src, v.edge_dst, v.edge_weight = _ptr(self.edge_src), _ptr(self.edge_dst), _ptr(self.edge_weight)
        v.num_edges = self.edge_src.size
        return v

    def nbytes(self) -> int:
        return sum(a.nbytes for a in (self.inserted, self.gt_ids, self.gt_labels, self.deleted, self.edge_src,
                                      self.edge_dst, self.edge_weight))


class Problem:
    """Seeded synthetic input: full CSR graph, true labels and the batch list,
    identical to the reference generator's output for the same arguments.

    cache_dir (default: the DLP_INPUT_CACHE environment variable; none when
    unset or empty) keeps the generated problem in a binary file there, keyed
    by the arguments, and reads it back on the next construction instead of
    generating again (dlp_problem_generate_cached). `from_cache` says which
    happened. Problem.load(path) reads such a file directly."""

    def __init__(self, num_nodes: int, avg_degree: int, num_batches: int, seed: int = 42,
                 gt_fraction: float = 0.01, deleted_fraction: float = 0.09, cache_dir: str | None = None):
        L = _n.lib()
        h = ctypes.c_void_p()
        cache_dir = os.environ.get("DLP_INPUT_CACHE") if cache_dir is None else cache_dir
        self.from_cache = False
        if cache_dir:
            Path(cache_dir).mkdir(parents=True, exist_ok=True)
            hit = ctypes.c_int(0)
            _n.check(L.dlp_problem_generate_cached(num_nodes, avg_degree, num_batches, seed, gt_fraction,
                                                   deleted_fraction, str(cache_dir).encode(), ctypes.byref(h),
                                                   ctypes.byref(hit)))
            self.from_cache = bool(hit.value)
        else:
            _n.check(L.dlp_problem_generate(num_nodes, avg_degree, num_batches, seed, gt_fraction,
                                            deleted_fraction, ctypes.byref(h)))
        self._take(h)

    @classmethod
    def load(cls, path: str | os.PathLike) -> "Problem":
        """A problem read from a cache file (dlp_problem_load: size and hash checked)."""
        L = _n.lib()
        h = ctypes.c_void_p()
        _n.check(L.dlp_problem_load(str(path).encode(), ctypes.byref(h)))
        self = cls.__new__(cls)
        self.from_cache = True
        self._take(h)
        return self

    def _take(self, h: ctypes.c_void_p) -> None:
        L = _n.lib()
        try:
            self.num_nodes = L.dlp_problem_num_nodes(h)
            m = L.dlp_problem_num_edges(h)
            n = self.num_nodes
            cp = lambda p, cnt, t: np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(t)), (cnt,)).copy() \
                if cnt else np.zeros(0, dtype=np.dtype(t))
            self.row_ptr = cp(L.dlp_problem_row_ptr(h), n + 1, ctypes.c_int32)
            self.col_ind = cp(L.dlp_problem_col_ind(h), m, ctypes.c_int32)
            self.values = cp(L.dlp_problem_values(h), m, ctypes.c_float)
            self.true_labels = cp(L.dlp_problem_true_labels(h), n, ctypes.c_float)
            self.batches: list[Batch] = []
            for b in range(L.dlp_problem_num_batches(h)):
                v = _n.BatchView()
                _n.check(L.dlp_problem_batch(h, b, ctypes.byref(v)))
                self.batches.append(Batch(
                    cp(v.inserted, v.num_inserted, ctypes.c_int32), cp(v.gt_ids, v.num_gt, ctypes.c_int32),
                    cp(v.gt_labels, v.num_gt, ctypes.c_float), cp(v.deleted, v.num_deleted, ctypes.c_int32),
                    cp(v.edge_src, v.num_edges, ctypes.c_int32), cp(v.edge_dst, v.num_edges, ctypes.c_int32),
                    cp(v.edge_weight, v.num_edges, ctypes.c_float)))
        finally:
            L.dlp_problem_free(h)

    @property
    def num_edges(self) -> int:
        return int(self.col_ind.size)

    def batch_map(self) -> np.ndarray:
        return batch_map(self.num_nodes, self.batches)


def batch_map(num_nodes: int, batches: list[Batch]) -> np.ndarray:
    """Batch of (last) arrival per vertex, -1 if never (src/dynLP.cu:193-198)."""
    m = np.full(num_nodes, -1, dtype=np.int32)
    for b, bt in enumerate(batches):
        m[bt.inserted] = b
    return m


@dataclass
class IrlpSnapshot:
    """The IrLP full-recompute input for the graph as it stands after a batch."""
    row_ptr: np.ndarray      # int32, n + 1: active rows, active neighbours, in CSR order
    col_ind: np.ndarray      # int32
    values: np.ndarray       # float32
    status: np.ndarray       # int32 per vertex: 0 active, 1 deleted (or not yet inserted), 2 ground truth
    gt_class: np.ndarray     # int32 per vertex: 0 / 1 for ground truth, -1 otherwise
    labels: np.ndarray       # float32 per vertex: the ground-truth label, 0.5 otherwise

    @property
    def num_nodes(self) -> int:
        return int(self.status.size)


def irlp_snapshot(p: "Problem", last_batch: int | None = None) -> IrlpSnapshot:
    """The snapshot the reference's driver hands to its IrLP baseline
    (src/main.cu:127-176), after batch `last_batch` (default: the last one):
    every vertex starts deleted; batch by batch, inserted vertices become
    active, deleted ones deleted, ground-truth ones ground truth with their
    class and label; the CSR keeps, for each live inserted vertex, its live
    inserted neighbours in the full graph's order."""
    n = p.num_nodes
    upto = len(p.batches) if last_batch is None else last_batch + 1
    status = np.full(n, 1, np.int32)
    gt = np.full(n, -1, np.int32)
    lab = np.full(n, 0.5, np.float32)
    inserted = np.zeros(n, bool)
    for bt in p.batches[:upto]:
        status[bt.inserted] = 0
        inserted[bt.inserted] = True
        status[bt.deleted] = 1
        status[bt.gt_ids] = 2
        gt[bt.gt_ids] = np.where(bt.gt_labels < 0.5, 0, 1)
        lab[bt.gt_ids] = bt.gt_labels
    live = (status != 1) & inserted
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(p.row_ptr).astype(np.int64))
    col = p.col_ind
    keep = live[rows] & (col >= 0)
    keep[keep] &= live[col[keep]]
    counts = np.bincount(rows[keep], minlength=n)
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    return IrlpSnapshot(row_ptr.astype(np.int32), col[keep].astype(np.int32), p.values[keep].astype(np.float32),
                        status, gt, lab)


def irlp(snap: IrlpSnapshot, delta: float = 1e-4, max_iterations: int = 100000, device: int = 0,
         timing: dict | None = None) -> tuple[np.ndarray, int]:
    """IrLP full recompute on the GPU (dlp_irlp, one cooperative launch; the
    reference's launchIrLP, src/validation.cu:145-208). Returns the labels and
    the iterations used. With `timing`, timing["ms"] is the launch's wall
    time, device synchronised on both sides, inputs already on the device."""
    L = _n.lib()
    _n.check(L.dlp_set_device(device))
    d = [DeviceArray(x) for x in (snap.row_ptr, snap.col_ind, snap.values, snap.labels, snap.status,
                                  snap.gt_class)]
    it = ctypes.c_int(0)
    _n.check(L.dlp_device_synchronize())
    t0 = time.perf_counter()
    _n.check(L.dlp_irlp(d[0].ptr, d[1].ptr, d[2].ptr, d[3].ptr, d[4].ptr, d[5].ptr, snap.num_nodes,
                        ctypes.c_float(delta), max_iterations, ctypes.byref(it), None))
    _n.check(L.dlp_device_synchronize())
    if timing is not None:
        timing["ms"] = 1e3 * (time.perf_counter() - t0)
    return d[3].get(), it.value


class Session:
    """One dynamic graph resident on the GPU (dlp_session_*)."""

    def __init__(self, num_nodes: int, row_ptr, col_ind, values, true_labels=None, vertex_batch_map=None, *,
                 tau: float = -1.0, delta: float = 1e-4, max_iterations: int = 100000,
                 semantics: int = SEMANTICS_REF, device: int = 0, record: bool = False, narrow_lanes: int = 0,
                 blocks_per_sm: int = 0, wait_timeout_s: float = 2.0, small_frontier_solo: int = 7,
                 solo_entry: int = 0, subgrid_entry: int = 0, arithmetic: int = 0):
        L = _n.lib()
        cfg = _n.Config()
        L.dlp_config_default(ctypes.byref(cfg))
        cfg.tau, cfg.delta, cfg.max_iterations = tau, delta, max_iterations
        cfg.semantics, cfg.device, cfg.record = semantics, device, int(bool(record))
        cfg.narrow_lanes, cfg.blocks_per_sm, cfg.wait_timeout_s = narrow_lanes, blocks_per_sm, wait_timeout_s
        cfg.small_frontier_solo = int(small_frontier_solo)
        cfg.solo_entry, cfg.subgrid_entry = int(solo_entry), int(subgrid_entry)
        cfg.arithmetic = int(arithmetic)
        self._keep = [np.ascontiguousarray(row_ptr, dtype=np.int32), np.ascontiguousarray(col_ind, dtype=np.int32),
                      np.ascontiguousarray(values, dtype=np.float32)]
        tl = None if true_labels is None else np.ascontiguousarray(true_labels, dtype=np.float32)
        bm = None if vertex_batch_map is None else np.ascontiguousarray(vertex_batch_map, dtype=np.int32)
        self.num_nodes = num_nodes
        self._h = ctypes.c_void_p()
        _n.check(L.dlp_session_create(ctypes.byref(cfg), num_nodes, self._keep[1].size, self._keep[0].ctypes.data,
                                      _ptr(self._keep[1]), _ptr(self._keep[2]), _ptr(tl), _ptr(bm),
                                      ctypes.byref(self._h)))
        self._keep = None

    @classmethod
    def from_problem(cls, p: Problem, **kw) -> "Session":
        return cls(p.num_nodes, p.row_ptr, p.col_ind, p.values, p.true_labels, p.batch_map(), **kw)

    def close(self) -> None:
        if self._h:
            _n.lib().dlp_session_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def tau(self) -> float:
        return float(_n.lib().dlp_session_tau(self._h))

    def reset(self) -> None:
        _n.check(_n.lib().dlp_session_reset(self._h))

    def apply(self, batch_index: int, batch: Batch, wait: bool = True) -> dict | None:
        v = batch.view()
        if wait:
            st = _n.BatchStats()
            _n.check(_n.lib().dlp_session_apply_batch(self._h, batch_index, ctypes.byref(v), ctypes.byref(st)))
            return st.as_dict()
        _n.check(_n.lib().dlp_session_apply_batch(self._h, batch_index, ctypes.byref(v), None))
        return None

    def apply_device(self, batch_index: int, dbatch: "DeviceBatch") -> None:
        v = dbatch.view()
        _n.check(_n.lib().dlp_session_apply_batch_device(self._h, batch_index, ctypes.byref(v)))

    def synchronize(self) -> None:
        _n.check(_n.lib().dlp_session_synchronize(self._h))

    def stats(self, batch_index: int) -> dict:
        st = _n.BatchStats()
        _n.check(_n.lib().dlp_session_stats(self._h, batch_index, ctypes.byref(st)))
        return st.as_dict()

    def elapsed_ms(self, first: int, last: int) -> float:
        ms = ctypes.c_float(0.0)
        _n.check(_n.lib().dlp_session_elapsed_ms(self._h, first, last, ctypes.byref(ms)))
        return float(ms.value)

    def pass_modes(self) -> dict:
        """Propagation passes so far by mode and their device seconds."""
        p = (ctypes.c_ulonglong * 4)()
        t = (ctypes.c_double * 4)()
        _n.check(_n.lib().dlp_session_pass_modes(self._h, p, t))
        names = ("one_block", "team", "sub_grid", "full_grid")
        return {n: {"passes": int(p[i]), "seconds": float(t[i])} for i, n in enumerate(names)}

    def debug(self) -> dict:
        out = (ctypes.c_int * 4)()
        _n.check(_n.lib().dlp_session_debug(self._h, out))
        return {"err": out[0], "phase": out[1], "pass": out[2], "small_passes": out[3]}

    def labels(self) -> np.ndarray:
        out = np.empty(self.num_nodes, dtype=np.float32)
        _n.check(_n.lib().dlp_session_read_labels(self._h, out.ctypes.data))
        return out

    def artefact(self, which: int) -> np.ndarray:
        cnt = ctypes.c_int64(0)
        _n.check(_n.lib().dlp_session_artefact(self._h, which, None, 0, ctypes.byref(cnt)))
        dt = np.float32 if which in (_n.ART_INIT_LABELS, _n.ART_LABELS) else np.int32
        out = np.empty(cnt.value, dtype=dt)
        if cnt.value:
            _n.check(_n.lib().dlp_session_artefact(self._h, which, out.ctypes.data, cnt.value, ctypes.byref(cnt)))
        return out


class Engine:
    """Many resident graphs; step() applies one batch to each of several graphs
    in one cooperative launch (dlp_engine_*)."""

    def __init__(self, max_graphs: int, memory_budget_bytes: int = 0, *, tau: float = -1.0, delta: float = 1e-4,
                 max_iterations: int = 100000, semantics: int = SEMANTICS_REF, device: int = 0, record: bool = False,
                 narrow_lanes: int = 0, blocks_per_sm: int = 0, wait_timeout_s: float = 2.0,
                 small_frontier_solo: int = 7, solo_entry: int = 0, subgrid_entry: int = 0,
                 arithmetic: int = 0):
        L = _n.lib()
        cfg = _n.Config()
        L.dlp_config_default(ctypes.byref(cfg))
        cfg.tau, cfg.delta, cfg.max_iterations = tau, delta, max_iterations
        cfg.semantics, cfg.device, cfg.record = semantics, device, int(bool(record))
        cfg.narrow_lanes, cfg.blocks_per_sm, cfg.wait_timeout_s = narrow_lanes, blocks_per_sm, wait_timeout_s
        cfg.small_frontier_solo = int(small_frontier_solo)
        cfg.solo_entry, cfg.subgrid_entry = int(solo_entry), int(subgrid_entry)
        cfg.arithmetic = int(arithmetic)
        self._h = ctypes.c_void_p()
        _n.check(L.dlp_engine_create(ctypes.byref(cfg), max_graphs, memory_budget_bytes, ctypes.byref(self._h)))
        self.sizes: dict[int, int] = {}
        import weakref
        self._servers = weakref.WeakSet()  # a server must be destroyed before its engine

    @staticmethod
    def graph_bytes(num_nodes: int, num_edges: int, truth: bool = True, batch_map: bool = True,
                    record: bool = False) -> int:
        return int(_n.lib().dlp_engine_graph_bytes(num_nodes, num_edges, int(truth), int(batch_map), int(record)))

    @property
    def bytes_in_use(self) -> int:
        return int(_n.lib().dlp_engine_bytes_in_use(self._h))

    def add_graph(self, num_nodes, row_ptr, col_ind, values, true_labels=None, vertex_batch_map=None) -> int:
        keep = [np.ascontiguousarray(row_ptr, dtype=np.int32), np.ascontiguousarray(col_ind, dtype=np.int32),
                np.ascontiguousarray(values, dtype=np.float32)]
        tl = None if true_labels is None else np.ascontiguousarray(true_labels, dtype=np.float32)
        bm = None if vertex_batch_map is None else np.ascontiguousarray(vertex_batch_map, dtype=np.int32)
        gid = ctypes.c_int(-1)
        _n.check(_n.lib().dlp_engine_add_graph(self._h, num_nodes, keep[1].size, keep[0].ctypes.data, _ptr(keep[1]),
                                               _ptr(keep[2]), _ptr(tl), _ptr(bm), ctypes.byref(gid)))
        self.sizes[gid.value] = num_nodes
        return gid.value

    def add_problem(self, p: Problem) -> int:
        return self.add_graph(p.num_nodes, p.row_ptr, p.col_ind, p.values, p.true_labels, p.batch_map())

    def remove_graph(self, gid: int) -> None:
        _n.check(_n.lib().dlp_engine_remove_graph(self._h, gid))
        self.sizes.pop(gid, None)

    def reset_graph(self, gid: int) -> None:
        _n.check(_n.lib().dlp_engine_reset_graph(self._h, gid))

    def snapshot(self, gid: int) -> bytes:
        """The graph's whole device state as bytes (for eviction)."""
        L = _n.lib()
        size = ctypes.c_size_t(0)
        _n.check(L.dlp_engine_snapshot(self._h, gid, None, 0, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        _n.check(L.dlp_engine_snapshot(self._h, gid, buf, size.value, ctypes.byref(size)))
        return buf.raw

    def restore(self, snap: bytes) -> int:
        """Makes a snapshotted graph resident again; returns its id."""
        gid = ctypes.c_int(-1)
        _n.check(_n.lib().dlp_engine_restore(self._h, snap, len(snap), ctypes.byref(gid)))
        self.sizes[gid.value] = int(_n.lib().dlp_engine_graph_nodes(self._h, gid.value))
        return gid.value

    def restore_as(self, snap: bytes, gid: int) -> None:
        """Makes a snapshotted graph resident again under the given free id."""
        _n.check(_n.lib().dlp_engine_restore_as(self._h, snap, len(snap), gid))
        self.sizes[gid] = int(_n.lib().dlp_engine_graph_nodes(self._h, gid))

    def tau(self, gid: int) -> float:
        return float(_n.lib().dlp_engine_tau(self._h, gid))

    def step(self, items: list[tuple[int, int, "Batch"]], wait: bool = True):
        """items: (graph id, batch index, Batch with host arrays)."""
        n = len(items)
        gids = (ctypes.c_int * n)(*[g for g, _, _ in items])
        bidx = (ctypes.c_int * n)(*[b for _, b, _ in items])
        views = (_n.BatchView * n)(*[bt.view() for _, _, bt in items])
        if wait:
            stats = (_n.BatchStats * n)()
            _n.check(_n.lib().dlp_engine_step(self._h, n, gids, bidx, views, stats))
            return [s.as_dict() for s in stats]
        _n.check(_n.lib().dlp_engine_step(self._h, n, gids, bidx, views, None))
        return None

    def step_device(self, items: list[tuple[int, int, "DeviceBatch"]]) -> None:
        n = len(items)
        gids = (ctypes.c_int * n)(*[g for g, _, _ in items])
        bidx = (ctypes.c_int * n)(*[b for _, b, _ in items])
        views = (_n.BatchView * n)(*[db if isinstance(db, _n.BatchView) else db.view() for _, _, db in items])
        _n.check(_n.lib().dlp_engine_step_device(self._h, n, gids, bidx, views))

    def step_sliced(self, items: list[tuple[int, int, "DeviceBatch"]], pass_budget: int = 0,
                    slice_us: float = 0.0) -> tuple[list[int], int]:
        """Starts the given batches (device arrays that must outlive their batch)
        and continues every unfinished one, for at most pass_budget passes /
        slice_us of propagation. Returns (graphs whose batch ended, graphs still
        in progress)."""
        n = len(items)
        gids = (ctypes.c_int * max(n, 1))(*[g for g, _, _ in items])
        bidx = (ctypes.c_int * max(n, 1))(*[b for _, b, _ in items])
        views = (_n.BatchView * max(n, 1))(*[db if isinstance(db, _n.BatchView) else db.view() for _, _, db in items])
        fin = (ctypes.c_int * 1024)()
        nf, nc = ctypes.c_int(0), ctypes.c_int(0)
        _n.check(_n.lib().dlp_engine_step_sliced(self._h, n, gids, bidx, views, pass_budget, slice_us, fin,
                                                 ctypes.byref(nf), ctypes.byref(nc)))
        return [fin[i] for i in range(nf.value)], nc.value

    def reserve(self, gid: int, max_edges: int, max_deleted: int) -> None:
        _n.check(_n.lib().dlp_engine_reserve(self._h, gid, max_edges, max_deleted))

    def in_progress(self, gid: int) -> bool:
        return bool(_n.lib().dlp_engine_in_progress(self._h, gid))

    def synchronize(self) -> None:
        _n.check(_n.lib().dlp_engine_synchronize(self._h))

    def stats(self, gid: int, batch_index: int) -> dict:
        st = _n.BatchStats()
        _n.check(_n.lib().dlp_engine_stats(self._h, gid, batch_index, ctypes.byref(st)))
        return st.as_dict()

    def debug(self) -> dict:
        out = (ctypes.c_int * 4)()
        _n.check(_n.lib().dlp_engine_debug(self._h, out))
        return {"err": out[0], "phase": out[1], "pass": out[2], "small_passes": out[3]}

    @property
    def steps(self) -> int:
        return int(_n.lib().dlp_engine_steps(self._h))

    def pass_modes(self) -> dict:
        """Propagation passes so far by mode and their device seconds."""
        p = (ctypes.c_ulonglong * 4)()
        t = (ctypes.c_double * 4)()
        _n.check(_n.lib().dlp_engine_pass_modes(self._h, p, t))
        names = ("one_block", "team", "sub_grid", "full_grid")
        return {n: {"passes": int(p[i]), "seconds": float(t[i])} for i, n in enumerate(names)}

    def elapsed_ms(self, first_step: int, last_step: int) -> float:
        ms = ctypes.c_float(0.0)
        _n.check(_n.lib().dlp_engine_elapsed_ms(self._h, first_step, last_step, ctypes.byref(ms)))
        return float(ms.value)

    def labels(self, gid: int) -> np.ndarray:
        out = np.empty(self.sizes[gid], dtype=np.float32)
        _n.check(_n.lib().dlp_engine_read_labels(self._h, gid, out.ctypes.data))
        return out

    def close(self) -> None:
        if self._h:
            for srv in list(self._servers):
                srv.close()
            _n.lib().dlp_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(sizes: list[int], degrees: list[int], batches: int = 10, max_iterations: int = 2000,
             **config) -> dict:
    """Times every launch-shape candidate (lanes per short row x one-block
    and sub-grid frontier thresholds x blocks per SM) on a generated sample of
    the given graph sizes and degrees and returns the fastest as
    {"narrow_lanes", "blocks_per_sm", "engine_kw": {solo_entry, subgrid_entry},
    "candidates"}; every candidate gave the same statistics (checked by the
    library)."""
    L = _n.lib()
    cfg = _n.Config()
    L.dlp_config_default(ctypes.byref(cfg))
    for k, v in config.items():
        setattr(cfg, k, v)
    n = len(sizes)
    sz = (ctypes.c_int * n)(*sizes)
    dg = (ctypes.c_int * n)(*degrees)
    rep = _n.TuneReport()
    _n.check(L.dlp_autotune(ctypes.byref(cfg), n, sz, dg, batches, max_iterations, ctypes.byref(rep)))
    cands = [{"narrow_lanes": rep.lanes[i], "blocks_per_sm": rep.blocks_per_sm[i], "solo_entry": rep.solo_entry[i],
              "subgrid_entry": rep.subgrid_entry[i], "ms": rep.ms[i]} for i in range(rep.candidates)]
    return {"narrow_lanes": cfg.narrow_lanes, "blocks_per_sm": cfg.blocks_per_sm,
            "engine_kw": {"solo_entry": cfg.solo_entry, "subgrid_entry": cfg.subgrid_entry}, "candidates": cands}


def device_name(device: int = 0) -> str:
    buf = ctypes.create_string_buffer(256)
    _n.check(_n.lib().dlp_device_name(device, buf, 256))
    return buf.value.decode()


def _kernel_digest() -> str:
    """Digest of the engine kernel's sources: a tuned shape is only reused for
    the kernel it was measured on."""
    import hashlib
    from pathlib import Path
    h = hashlib.sha256()
    for name in ("engine_kernel.cu", "engine.cuh", "row_sums.cuh", "session_kernel.cuh", "tune.cu"):
        f = Path(__file__).resolve().parent / "csrc" / name
        if f.exists():
            h.update(f.read_bytes())
    return h.hexdigest()[:16]


def autotune_cached(sizes: list[int], degrees: list[int], batches: int = 10, max_iterations: int = 2000,
                    cache_path: str | None = None, **config) -> dict:
    """autotune() with a JSON cache keyed by GPU model and engine-kernel
    digest (DLP_TUNE_CACHE, default ~/.cache/dlp_gb300/tune.json): a GPU model
    is tuned once per kernel version and the choice is reused after that.
    The result says where it came from ("source": "cache" or "measured")."""
    import json
    import os
    from pathlib import Path
    path = Path(cache_path or os.environ.get("DLP_TUNE_CACHE") or
                Path.home() / ".cache" / "dlp_gb300" / "tune.json")
    key = f"{device_name(config.get('device', 0))} | kernel {_kernel_digest()} | " \
          f"sizes {sorted(sizes)} degrees {sorted(degrees)} batches {batches} max_iter {max_iterations}"
    try:
        cache = json.loads(path.read_text())
    except (OSError, ValueError):
        cache = {}
    if key in cache:
        return dict(cache[key], source="cache", key=key)
    r = autotune(sizes, degrees, batches=batches, max_iterations=max_iterations, **config)
    cache[key] = r
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        tmp.replace(path)
    except OSError:
        pass
    return dict(r, source="measured", key=key)


class Server:
    """Continuous batching over an Engine (dlp_server_*): requests wait in
    arrival order; each poll admits what fits and runs one sliced step over the
    admitted batches and those in progress. serial=True is the plain path."""

    def __init__(self, engine: Engine, *, slice_us: float = 2000.0, pass_budget: int = 0,
                 memory_budget_bytes: int = 0, max_batches_per_step: int = 0, serial: bool = False,
                 evict_idle: bool = False):
        L = _n.lib()
        cfg = _n.ServerConfig()
        L.dlp_server_config_default(ctypes.byref(cfg))
        cfg.slice_us, cfg.pass_budget = slice_us, pass_budget
        cfg.memory_budget_bytes, cfg.max_batches_per_step, cfg.serial = memory_budget_bytes, max_batches_per_step, \
            int(bool(serial))
        cfg.evict_idle = int(bool(evict_idle))
        self.engine = engine
        self._h = ctypes.c_void_p()
        _n.check(L.dlp_server_create(engine._h, ctypes.byref(cfg), ctypes.byref(self._h)))
        engine._servers.add(self)

    def reserve(self, gid: int, batches: list[Batch]) -> None:
        """Sizes the graph's buffers for the largest of the given batches."""
        m = lambda f: max((f(b) for b in batches), default=0)
        _n.check(_n.lib().dlp_server_reserve(self._h, gid, m(lambda b: b.inserted.size), m(lambda b: b.gt_ids.size),
                                             m(lambda b: b.deleted.size), m(lambda b: b.edge_src.size)))

    def submit(self, gid: int, batch_index: int, batch: Batch) -> int:
        req = _n.Request(gid, batch_index, batch.view(), 0.0)
        rid = ctypes.c_int(-1)
        _n.check(_n.lib().dlp_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)))
        return rid.value

    def poll(self) -> list[int]:
        ids = (ctypes.c_int * 4096)()
        nc = ctypes.c_int(0)
        _n.check(_n.lib().dlp_server_poll(self._h, ids, 4096, ctypes.byref(nc)))
        return [ids[i] for i in range(min(nc.value, 4096))]

    @property
    def pending(self) -> int:
        return int(_n.lib().dlp_server_pending(self._h))

    def evictions(self) -> tuple[int, int]:
        """(graphs evicted to host memory, graphs restored) so far."""
        ev, rs = ctypes.c_int(0), ctypes.c_int(0)
        _n.check(_n.lib().dlp_server_evictions(self._h, ctypes.byref(ev), ctypes.byref(rs)))
        return ev.value, rs.value

    def make_resident(self, gid: int) -> None:
        _n.check(_n.lib().dlp_server_make_resident(self._h, gid))

    def drain(self) -> list[int]:
        done = []
        while self.pending:
            done += self.poll()
        return done

    def result(self, rid: int) -> dict:
        r = _n.RequestResult()
        _n.check(_n.lib().dlp_server_result(self._h, rid, ctypes.byref(r)))
        return _result_dict(r)

    def replay(self, trace: list[tuple[float, int, int, Batch]]) -> tuple[list[dict], float]:
        """trace: (arrival seconds, graph id, batch index, Batch), sorted by
        arrival. Returns per-request results and the makespan in seconds."""
        n = len(trace)
        reqs = (_n.Request * max(n, 1))()
        for i, (t, g, b, bt) in enumerate(trace):
            reqs[i] = _n.Request(g, b, bt.view(), t)
        out = (_n.RequestResult * max(n, 1))()
        span = ctypes.c_double(0.0)
        _n.check(_n.lib().dlp_server_replay(self._h, n, reqs, out, ctypes.byref(span)))
        return [_result_dict(out[i]) for i in range(n)], float(span.value)

    def close(self) -> None:
        """Destroys the server (before its engine: destroying restores the
        graphs it evicted into the engine)."""
        if self._h:
            if self.engine._h:
                _n.lib().dlp_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _result_dict(r) -> dict:
    return {"graph_id": r.graph_id, "batch_index": r.batch_index, "status": r.status, "arrival_s": r.arrival_s,
            "admit_s": r.admit_s, "finish_s": r.finish_s, "steps": r.steps, "stats": r.stats.as_dict()}


class DeviceArray:
    """A device buffer owned by Python (dlp_malloc / dlp_free)."""

    def __init__(self, host: np.ndarray | None = None, *, nbytes: int | None = None, dtype=None, count=None):
        L = _n.lib()
        if host is not None:
            host = np.ascontiguousarray(host)
            self.dtype, self.count, nbytes = host.dtype, host.size, host.nbytes
        else:
            self.dtype = np.dtype(dtype) if dtype is not None else np.dtype(np.uint8)
            self.count = count if count is not None else nbytes // self.dtype.itemsize
            nbytes = self.count * self.dtype.itemsize
        self.nbytes = nbytes
        self.ptr = ctypes.c_void_p()
        _n.check(L.dlp_malloc(ctypes.byref(self.ptr), max(nbytes, 16)))
        if host is not None and nbytes:
            _n.check(L.dlp_memcpy_htod(self.ptr, host.ctypes.data, nbytes))

    @property
    def addr(self) -> int:
        return self.ptr.value or 0

    def get(self, dtype=None) -> np.ndarray:
        dt = np.dtype(dtype) if dtype is not None else self.dtype
        out = np.empty(self.nbytes // dt.itemsize, dtype=dt)
        if self.nbytes:
            _n.check(_n.lib().dlp_memcpy_dtoh(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def set(self, host: np.ndarray) -> None:
        """Copies the host array's bytes (no dtype conversion)."""
        host = np.ascontiguousarray(host)
        if host.nbytes > self.nbytes:
            raise ValueError("host array larger than the device buffer")
        _n.check(_n.lib().dlp_memcpy_htod(self.ptr, host.ctypes.data, host.nbytes))

    def free(self) -> None:
        if self.ptr:
            _n.lib().dlp_free(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PackedBatches:
    """Many batches uploaded to one device buffer with one copy (16-byte
    aligned segments); view(i) is the device view of batch i."""

    def __init__(self, batches: list[Batch]):
        parts, offs = [], []
        off = 0
        for bt in batches:
            o = []
            for a in (bt.inserted, bt.gt_ids, bt.gt_labels, bt.deleted, bt.edge_src, bt.edge_dst, bt.edge_weight):
                o.append(off)
                parts.append((off, a))
                off += (a.nbytes + 15) & ~15
            offs.append(o)
        host = np.zeros(max(off, 16), dtype=np.uint8)
        for o, a in parts:
            if a.nbytes:
                host[o:o + a.nbytes] = np.frombuffer(np.ascontiguousarray(a).tobytes(), dtype=np.uint8)
        self.buf = DeviceArray(host)
        self.offs = offs
        self.sizes = [(bt.inserted.size, bt.gt_ids.size, bt.deleted.size, bt.edge_src.size) for bt in batches]

    def view(self, i: int) -> _n.BatchView:
        base = self.buf.addr
        o = [base + x for x in self.offs[i]]
        ni, ng, nd, ne = self.sizes[i]
        v = _n.BatchView()
        v.inserted, v.num_inserted = o[0], ni
        v.gt_ids, v.gt_labels, v.num_gt = o[1], o[2], ng
        v.deleted, v.num_deleted = o[3], nd
        v.edge_src, v.edge_dst, v.edge_weight, v.num_edges = o[4], o[5], o[6], ne
        return v


class DeviceBatch:
    """A batch uploaded once to device memory (for device-resident replays)."""

    def __init__(self, batch: Batch):
        self.parts = [DeviceArray(a) for a in (batch.inserted, batch.gt_ids, batch.gt_labels, batch.deleted,
                                               batch.edge_src, batch.edge_dst, batch.edge_weight)]
        self.sizes = (batch.inserted.size, batch.gt_ids.size, batch.deleted.size, batch.edge_src.size)

    def view(self) -> _n.BatchView:
        p = [a.addr for a in self.parts]
        v = _n.BatchView()
        v.inserted, v.num_inserted = p[0], self.sizes[0]
        v.gt_ids, v.gt_labels, v.num_gt = p[1], p[2], self.sizes[1]
        v.deleted, v.num_deleted = p[3], self.sizes[2]
        v.edge_src, v.edge_dst, v.edge_weight, v.num_edges = p[4], p[5], p[6], self.sizes[3]
        return v
