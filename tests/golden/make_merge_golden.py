"""Generate the merge-stage fixtures by running the REFERENCE itself.

For every case in cases.MERGE_CASES the reference's node dump driver runs
with -d (oracle/ref_dump.cpp: the reference's own construction, cutoff,
simplifyDistNodeGraph and gatherDistNodeGraph, compiled from its sources
against the project's single-rank MPI shim). Stored next to this script:

  merge_cases.json        per case: the input hash, the SHA-256, size and line
                          count of the reference's contigGraph.txt
  <name>.order.npy        the reference's visiting order: for each node, in
                          the order its merge loop visits it (its node map's
                          iteration order, which nodes.txt is printed in), the
                          node's index among the k-molecules sorted by key

With the order the CPU restatement replays the reference's merge without the
reference. Run from the repository root where the reference tree exists:
    python tests/golden/make_merge_golden.py
"""
from __future__ import annotations

import hashlib
import json
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "swap-assembler_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(HERE))

import oracle  # noqa: E402

from cases import MERGE_CASES, case_text  # noqa: E402


def main() -> None:
    if not oracle.reference_available():
        sys.exit("the reference binaries (oracle/_ref) are not built")
    out = {}
    tmp = Path(tempfile.mkdtemp(prefix="swg_merge_golden_"))
    try:
        for case in MERGE_CASES:
            text = case_text(case)
            fa = tmp / (case["name"] + ".fa")
            fa.write_bytes(text)
            nodes, merged = oracle.run_reference_merge(str(fa), case["k"], case["c"],
                                                       str(tmp / case["name"]))
            keys, _ = oracle.parse_node_lines(nodes)
            order = np.argsort(np.argsort(keys, kind="stable"), kind="stable").astype(np.uint32)
            np.save(HERE / (case["name"] + ".order.npy"), order)
            out[case["name"]] = dict(
                k=case["k"], c=case["c"], why=case["why"],
                input_sha256=hashlib.sha256(text).hexdigest(),
                nodes=int(keys.size),
                merged_sha256=hashlib.sha256(merged).hexdigest(),
                merged_bytes=len(merged),
                merged_lines=merged.count(b"\n") - 1,
            )
            print(case["name"], out[case["name"]]["nodes"], out[case["name"]]["merged_lines"])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    (HERE / "merge_cases.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
