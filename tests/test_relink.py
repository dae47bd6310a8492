"""Drop-in checks: the reference's own driver and writers against this
repository's headers and library.

1. The reference's src/main.cu, unmodified, compiles against include/ and
   links against libdynlp_gb300.so (CPU: it must then stop cleanly at
   runDynLP with a device error).
2. On a GPU the same binary runs the reference's default small workload
   (5,000 vertices, 10 batches, seed 42) end to end; its dynlp_labels.txt and
   results.csv must hold exactly the oracle's labels and accuracies in the
   reference's text formats (src/utils.cu:161-200).
3. The library's writeLabelsToFile / writeResultsCSV write byte for byte what
   the reference's own writers (src/utils.cu:161-200, built from its sources
   into oracle/_ref/utils.o) write for the same arrays.

The reference's sources come from the guarded copy in oracle/_ref/src (made by
`make -C oracle refsrc`; main.cu and utils.cu are not changed by the guards)
or from the checkout named by DLP_REFERENCE_DIR. Where neither exists the
tests are skipped. Binaries are built in temporary directories.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
LIB_DIR = ROOT / "labelpropcuda_gb300" / "_build"
REF_UTILS_O = ROOT / "oracle" / "_ref" / "utils.o"
REF_HEADERS = ROOT / "oracle" / "_ref" / "headers"


def reference_main() -> Path | None:
    for base in (ROOT / "oracle" / "_ref", Path(os.environ.get("DLP_REFERENCE_DIR", "/nonexistent"))):
        f = base / "src" / "main.cu"
        if f.exists():
            return f
    return None


NVCC = shutil.which("nvcc")
needs_main = pytest.mark.skipif(reference_main() is None or NVCC is None,
                                reason="reference sources (oracle/_ref/src) or nvcc not available")


def build_main(td: Path) -> Path:
    exe = td / "dynLP"
    subprocess.run([NVCC, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "--pre-include", "iomanip",
                    "-I", str(ROOT / "include"), str(reference_main()), "-o", str(exe), "-L", str(LIB_DIR),
                    "-ldynlp_gb300", "-Xlinker", f"-rpath={LIB_DIR}"], check=True, capture_output=True)
    return exe


@needs_main
def test_reference_main_relinks(native):
    with tempfile.TemporaryDirectory() as td:
        exe = build_main(Path(td))
        out = subprocess.run([str(exe), "--help"], capture_output=True, text=True)
        assert "--totalNodes" in out.stdout and "--noValidate" in out.stdout
        import labelpropcuda_gb300 as dlp
        if dlp.device_count() > 0:
            return  # the GPU run is test_reference_main_runs_on_gpu
        run = subprocess.run([str(exe), "--totalNodes", "2000", "--numBatches", "3", "--output", td, "--noValidate",
                              "--quiet"], capture_output=True, text=True, timeout=120)
        assert "Generated graph: 2000 nodes" in run.stdout
        assert (Path(td) / "graph" / "csrRowPtr.txt").exists()
        assert run.returncode == 1 and "DynLP execution failed" in run.stdout


@pytest.mark.gpu
@needs_main
def test_reference_main_runs_on_gpu(gpu, oracle):
    n, nb = 5000, 10
    with tempfile.TemporaryDirectory() as td:
        exe = build_main(Path(td))
        out = Path(td) / "out"
        run = subprocess.run([str(exe), "--totalNodes", str(n), "--numBatches", str(nb), "--output", str(out),
                              "--noValidate", "--quiet"], capture_output=True, text=True, timeout=600)
        assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-2000:]
        lab_lines = (out / "dynlp_labels.txt").read_text().splitlines()
        csv_lines = (out / "results.csv").read_text().splitlines()
    p = oracle.OracleProblem(n, 5, nb, 42)
    orc = oracle.OracleRun.from_problem(p, threads=0)
    accs = [orc.apply(b, bt)["accuracy"] for b, bt in enumerate(p.batches)]
    want = orc.labels()
    assert len(lab_lines) == n
    assert lab_lines == ["%d %.6f" % (i, float(x)) for i, x in enumerate(want)]
    assert csv_lines[0] == "batch,time_ms,accuracy"
    assert len(csv_lines) == nb + 1
    for b, ln in enumerate(csv_lines[1:]):
        idx, ms, acc = ln.split(",")
        assert int(idx) == b and float(ms) >= 0.0
        assert acc == "%.6f" % float(np.float32(accs[b]))


WRITER_DRIVER = r"""
#include <cstdlib>
#include <string>
#include <vector>
#include "utils.h"
int main(int argc, char **argv) {
  std::vector<float> lab = {0.0f, 1.0f, 0.5f, 1e-7f, 0.9999995f, 0.1234565f, 0.33333334f, 0.66666669f,
                            2.5e-6f, 0.5000005f, 0.49999997f, 0.7f};
  for (int i = 0; i < 2000; ++i) lab.push_back(static_cast<float>((i * 2654435761u) % 1000003u) / 1000003.0f);
  std::vector<float> ms = {0.0f, 1.005f, 12345.678f, 0.125f, 3.14159f};
  std::vector<float> acc = {0.0f, 1.0f, 0.5f, 0.99999994f, 0.1234565f};
  bool ok = writeLabelsToFile(std::string(argv[1]), lab.data(), static_cast<int>(lab.size()));
  ok = ok && writeResultsCSV(std::string(argv[2]), ms.data(), acc.data(), static_cast<int>(ms.size()));
  return ok ? 0 : 1;
}
"""


@pytest.mark.skipif(not REF_UTILS_O.exists() or NVCC is None,
                    reason="the reference's writers (oracle/_ref/utils.o) or nvcc not available")
def test_writers_byte_identical_to_reference(native):
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        drv = td / "drv.cu"
        drv.write_text(WRITER_DRIVER)
        ref_exe, our_exe = td / "ref_w", td / "our_w"
        subprocess.run([NVCC, "-std=c++17", "-I", str(REF_HEADERS), str(drv), str(REF_UTILS_O), "-o",
                        str(ref_exe)], check=True, capture_output=True)
        subprocess.run([NVCC, "-std=c++17", "-I", str(ROOT / "include"), str(drv), "-o", str(our_exe),
                        "-L", str(LIB_DIR), "-ldynlp_gb300", "-Xlinker", f"-rpath={LIB_DIR}"], check=True,
                       capture_output=True)
        for exe, tag in ((ref_exe, "ref"), (our_exe, "our")):
            subprocess.run([str(exe), str(td / f"{tag}_labels.txt"), str(td / f"{tag}_results.csv")], check=True,
                           capture_output=True)
        assert (td / "our_labels.txt").read_bytes() == (td / "ref_labels.txt").read_bytes()
        assert (td / "our_results.csv").read_bytes() == (td / "ref_results.csv").read_bytes()
