"""The binary input cache (dlp_problem_save / _load / _generate_cached): a
cached problem is the generated one array for array, and a damaged, truncated
or mismatched file is never used. CPU only: no device is touched."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp
from labelpropcuda_gb300 import _native as N

ARGS = (3000, 5, 6, 7)


def same(a: dlp.Problem, b: dlp.Problem) -> None:
    assert a.num_nodes == b.num_nodes
    for k in ("row_ptr", "col_ind", "values", "true_labels"):
        x, y = getattr(a, k), getattr(b, k)
        assert x.dtype == y.dtype and np.array_equal(x, y), k
    assert len(a.batches) == len(b.batches)
    for ba, bb in zip(a.batches, b.batches):
        for k in ("inserted", "gt_ids", "gt_labels", "deleted", "edge_src", "edge_dst", "edge_weight"):
            assert np.array_equal(getattr(ba, k), getattr(bb, k)), k


def cache_files(d) -> list:
    return sorted(p for p in os.listdir(d) if p.endswith(".bin"))


def test_cached_problem_equals_generated(native, tmp_path):
    ref = dlp.Problem(*ARGS, cache_dir="")
    first = dlp.Problem(*ARGS, cache_dir=str(tmp_path))
    assert not first.from_cache
    files = cache_files(tmp_path)
    assert len(files) == 1 and files[0].startswith("dlp_problem_n3000_d5_b6_s7_")
    second = dlp.Problem(*ARGS, cache_dir=str(tmp_path))
    assert second.from_cache
    same(ref, first)
    same(ref, second)
    same(ref, dlp.Problem.load(tmp_path / files[0]))
    # other generator arguments, another file
    other = dlp.Problem(*ARGS, gt_fraction=0.02, cache_dir=str(tmp_path))
    assert not other.from_cache and len(cache_files(tmp_path)) == 2
    assert other.batches[0].gt_ids.size != ref.batches[0].gt_ids.size


def test_environment_variable_selects_the_cache(native, tmp_path, monkeypatch):
    monkeypatch.setenv("DLP_INPUT_CACHE", str(tmp_path / "envcache"))
    a = dlp.Problem(*ARGS)
    b = dlp.Problem(*ARGS)
    assert not a.from_cache and b.from_cache
    same(a, b)


def test_damaged_files_are_regenerated(native, tmp_path):
    ref = dlp.Problem(*ARGS, cache_dir=str(tmp_path))
    path = tmp_path / cache_files(tmp_path)[0]
    raw = bytearray(path.read_bytes())
    # one flipped payload byte: the hash no longer matches
    raw[len(raw) // 2] ^= 0x40
    path.write_bytes(bytes(raw))
    with pytest.raises(dlp.DlpError, match="hash"):
        dlp.Problem.load(path)
    again = dlp.Problem(*ARGS, cache_dir=str(tmp_path))
    assert not again.from_cache
    same(ref, again)
    assert dlp.Problem(*ARGS, cache_dir=str(tmp_path)).from_cache  # the file was rewritten
    # truncated
    raw = path.read_bytes()
    path.write_bytes(raw[:-100])
    with pytest.raises(dlp.DlpError, match="size"):
        dlp.Problem.load(path)
    assert not dlp.Problem(*ARGS, cache_dir=str(tmp_path)).from_cache
    # not a cache file at all
    path.write_bytes(b"not a cache file" * 8)
    with pytest.raises(dlp.DlpError, match="not a problem cache file"):
        dlp.Problem.load(path)
    assert not dlp.Problem(*ARGS, cache_dir=str(tmp_path)).from_cache
    same(ref, dlp.Problem(*ARGS, cache_dir=str(tmp_path)))


def test_file_of_another_key_is_not_used(native, tmp_path):
    dlp.Problem(3000, 5, 6, 8, cache_dir=str(tmp_path))  # seed 8
    (src,) = cache_files(tmp_path)
    want = src.replace("_s8_", "_s7_")
    os.rename(tmp_path / src, tmp_path / want)
    p = dlp.Problem(*ARGS, cache_dir=str(tmp_path))  # seed 7: the renamed file's key differs
    assert not p.from_cache
    same(dlp.Problem(*ARGS, cache_dir=""), p)


def test_c_abi_save_and_load(native, tmp_path):
    L = N.lib()
    h = ctypes.c_void_p()
    N.check(L.dlp_problem_generate(2000, 3, 4, 11, ctypes.c_float(0.01), ctypes.c_float(0.09), ctypes.byref(h)))
    path = str(tmp_path / "p.bin").encode()
    try:
        N.check(L.dlp_problem_save(h, path))
    finally:
        L.dlp_problem_free(h)
    assert not [p for p in os.listdir(tmp_path) if ".tmp." in p]  # the temporary file was renamed
    loaded = dlp.Problem.load(tmp_path / "p.bin")
    same(dlp.Problem(2000, 3, 4, 11, cache_dir=""), loaded)
    # the saved file is the one generate_cached would have written
    p2 = dlp.Problem(2000, 3, 4, 11, cache_dir=str(tmp_path / "c"))
    (name,) = cache_files(tmp_path / "c")
    assert (tmp_path / "c" / name).read_bytes() == (tmp_path / "p.bin").read_bytes()
    same(loaded, p2)
    with pytest.raises(dlp.DlpError):
        dlp.Problem.load(tmp_path / "missing.bin")
    # the C entry point creates a missing cache directory (one level)
    h = ctypes.c_void_p()
    hit = ctypes.c_int(1)
    d = str(tmp_path / "fresh").encode()
    N.check(L.dlp_problem_generate_cached(2000, 3, 4, 11, ctypes.c_float(0.01), ctypes.c_float(0.09), d,
                                          ctypes.byref(h), ctypes.byref(hit)))
    L.dlp_problem_free(h)
    assert hit.value == 0 and cache_files(tmp_path / "fresh") == [name]
