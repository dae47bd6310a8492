"""Drop-in check: the reference's own driver (src/main.cu, unmodified) compiles
against this repository's headers and links against libdynlp_gb300.so.

Runs only where the reference checkout exists (it is not shipped with this
repository); the binary is built in a temporary directory and never kept.
Without a GPU the run must stop cleanly at runDynLP with a device error.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REFERENCE_MAIN = Path("/root/reference/src/main.cu")


@pytest.mark.skipif(not REFERENCE_MAIN.exists() or shutil.which("nvcc") is None,
                    reason="reference checkout or nvcc not available")
def test_reference_main_relinks(native):
    lib_dir = ROOT / "labelpropcuda_gb300" / "_build"
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "dynLP"
        subprocess.run(["nvcc", "-std=c++17", "-arch=sm_103a", "--pre-include", "iomanip", "-I", str(ROOT / "include"),
                        str(REFERENCE_MAIN), "-o", str(exe), "-L", str(lib_dir), "-ldynlp_gb300",
                        f"-Xlinker", f"-rpath={lib_dir}"], check=True, capture_output=True)
        out = subprocess.run([str(exe), "--help"], capture_output=True, text=True)
        assert "--totalNodes" in out.stdout and "--noValidate" in out.stdout
        run = subprocess.run([str(exe), "--totalNodes", "2000", "--numBatches", "3", "--output", td, "--noValidate",
                              "--quiet"], capture_output=True, text=True, timeout=120)
        assert "Generated graph: 2000 nodes" in run.stdout
        assert (Path(td) / "graph" / "csrRowPtr.txt").exists()
        import labelpropcuda_gb300 as dlp
        if dlp.device_count() == 0:
            assert run.returncode == 1 and "DynLP execution failed" in run.stdout
