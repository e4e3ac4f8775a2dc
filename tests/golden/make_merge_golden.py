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
reference. The same script stores, per case, the reference's tip and
low-coverage passes (oracle/ref_prune.cpp: masterTipsRemoval and
masterLowCoverageEdgeRemoval, graph.cpp:2194-2300) run on the complete merge
of the case (oracle.merge_text, deterministic):

  <name>.prune_order.npy  the order those passes visit the nodes (the node map's
                          iteration order after recvBufDistNodeGraph) as
                          indices of the complete merge's lines
  merge_cases.json        also the SHA-256 and size of the graph after the
                          tip pass and after the low-coverage pass

and the reference's masterSimplifyNodeGraph (oracle/ref_simplify.cpp,
graph.cpp:2089-2192) run on the restatement's tip pass over the complete
merge (every non-tip first, then the tips in key order — deterministic):

  <name>.simplify_order.npy  its visiting order as line indices of that input
  merge_cases.json           the SHA-256 and size of its output

Run from the repository root where the reference tree exists:
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
            full = oracle.merge_text(*oracle.records(text, case["k"], case["c"]), case["k"])
            mp = tmp / (case["name"] + ".merged.txt")
            mp.write_bytes(full)
            before, tips, low = oracle.run_reference_prune(str(mp), case["k"], case["c"],
                                                           str(tmp / (case["name"] + "_prune")))
            index = {l.split(b" ", 1)[0]: i for i, l in enumerate(l for l in full.split(b"\n") if l)}
            porder = np.array([index[l.split(b" ", 1)[0]] for l in before.split(b"\n") if l],
                              dtype=np.uint32)
            np.save(HERE / (case["name"] + ".prune_order.npy"), porder)
            out[case["name"]].update(
                tips_sha256=hashlib.sha256(tips).hexdigest(), tips_bytes=len(tips),
                lowcov_sha256=hashlib.sha256(low).hexdigest(), lowcov_bytes=len(low))
            tips_in, _ = oracle.prune_text(full, case["k"], oracle.PRUNE_TIPS,
                                           oracle.tips_last_order(full, case["k"]))
            tp = tmp / (case["name"] + ".tips.txt")
            tp.write_bytes(tips_in)
            sb, sa = oracle.run_reference_simplify(str(tp), case["k"], case["c"],
                                                   str(tmp / (case["name"] + "_simplify")))
            tindex = {l.split(b" ", 1)[0]: i for i, l in enumerate(l for l in tips_in.split(b"\n") if l)}
            sorder = np.array([tindex[l.split(b" ", 1)[0]] for l in sb.split(b"\n") if l], dtype=np.uint32)
            np.save(HERE / (case["name"] + ".simplify_order.npy"), sorder)
            out[case["name"]].update(simplify_sha256=hashlib.sha256(sa).hexdigest(), simplify_bytes=len(sa))
            print(case["name"], out[case["name"]]["nodes"], out[case["name"]]["merged_lines"],
                  tips.count(b"\n") - 1, low.count(b"\n") - 1)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    (HERE / "merge_cases.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
