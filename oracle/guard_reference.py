"""Test infrastructure, not product code.

Makes the guarded copy of the reference's sources that the reference-kernel
harness (oracle/ref_kernels.cu) is built from:

    python3 oracle/guard_reference.py <reference checkout> oracle/_ref

copies <checkout>/src/*.cu and <checkout>/headers/*.h to oracle/_ref/src and
oracle/_ref/headers (git-ignored; never committed), then changes exactly three
statements of src/connectedComponents.cu. The reference reads and writes
index -1 there when a new vertex's tree reaches a vertex that is not new in
the batch (its parent array starts at -1 for those, :178):
  * jumpKernel reads par[-1]                 (:114-115)
  * markRootsKernel writes isRoot[-1]        (:136)
  * assignComponentIdsKernel reads rootToId[-1] (:155)
Each access is guarded with the convention the oracle pins: par[-1] reads -1,
the isRoot[-1] write is dropped, rootToId[-1] reads -1. Nothing else in the
copy changes. The reference's other out-of-bounds read (the components step
hooks numSubEdges entries of an edge list that holds numNewEdges, which can be
fewer: src/dynLP.cu:437-440) is bounded by the harness at the call, without a
source change.

Each guard is located by the statement it replaces, which must occur exactly
once in the file; the script fails when the reference has changed.
"""
from __future__ import annotations

import re
import shutil
import sys
from pathlib import Path

# (kernel, regex of the statement, replacement with the same variables)
GUARDS = [
    ("jumpKernel",
     r"int\s+grandparent\s*=\s*d_par\[parent\];",
     "int grandparent = parent < 0 ? -1 : d_par[parent];"),
    ("markRootsKernel",
     r"d_isRoot\[root\]\s*=\s*1;",
     "if (root >= 0) d_isRoot[root] = 1;"),
    ("assignComponentIdsKernel",
     r"d_componentId\[v\]\s*=\s*d_rootToId\[root\];",
     "d_componentId[v] = root < 0 ? -1 : d_rootToId[root];"),
]


def guard(text: str) -> str:
    for kernel, pattern, repl in GUARDS:
        hits = re.findall(pattern, text)
        if len(hits) != 1:
            raise SystemExit(f"guard for {kernel}: expected one match, found {len(hits)}")
        text = re.sub(pattern, lambda _m, r=repl: r, text, count=1)
    return text


def main(argv: list[str]) -> int:
    if len(argv) != 3:
        print(__doc__, file=sys.stderr)
        return 2
    ref, out = Path(argv[1]), Path(argv[2])
    if not (ref / "src" / "connectedComponents.cu").exists():
        print(f"{ref} is not a reference checkout", file=sys.stderr)
        return 2
    for sub, pat in (("src", "*.cu"), ("headers", "*.h")):
        (out / sub).mkdir(parents=True, exist_ok=True)
        for f in sorted((ref / sub).glob(pat)):
            shutil.copyfile(f, out / sub / f.name)
    cc = out / "src" / "connectedComponents.cu"
    cc.write_text(guard(cc.read_text()))
    (out / "src" / ".guarded").write_text("guards: " + ", ".join(g[0] for g in GUARDS) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
