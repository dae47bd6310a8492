"""The C-ABI library loads without a GPU and exports every symbol the public
headers declare; calls that need a device fail with a status, not a crash."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_c_functions() -> list[str]:
    text = (ROOT / "include" / "dlp_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dlp_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_function_is_exported(native):
    names = declared_c_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_binding_covers_header(native):
    from labelpropcuda_gb300 import _native as N
    assert set(declared_c_functions()) <= set(N.exported_symbols())


def test_abi_version_and_strings(native):
    assert native.dlp_abi_version() == 1
    assert native.dlp_status_string(4) == b"DLP_ERR_TIMEOUT"


def test_problem_generation_without_gpu(native):
    import labelpropcuda_gb300 as dlp
    p = dlp.Problem(1000, 3, 5, 7)
    assert p.row_ptr[-1] == p.col_ind.size == 3000
    assert len(p.batches) == 5


def test_invalid_generation_arguments(native):
    import labelpropcuda_gb300 as dlp
    with pytest.raises(dlp.DlpError):
        dlp.Problem(1, 3, 5, 7)
    with pytest.raises(dlp.DlpError):
        dlp.Problem(100, 3, 5, 7, gt_fraction=1.5)


def test_session_without_device_reports_status(native):
    import labelpropcuda_gb300 as dlp
    if dlp.device_count() > 0:
        pytest.skip("a device is present")
    p = dlp.Problem(1000, 3, 5, 7)
    with pytest.raises(dlp.DlpError) as e:
        dlp.Session.from_problem(p)
    assert e.value.status in (5, 2)
