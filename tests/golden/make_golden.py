"""Generate the golden fixtures by running the REFERENCE itself.

The reference ships no tests or golden vectors, so the fixtures here are the
reference's own outputs on project-written inputs: the unmodified `swap -s`
(kmerGraph.txt) and the node dump driver (every surviving k-molecule with its
8 multiplicities), both compiled from the reference's sources by
oracle/Makefile against the project's single-rank MPI shim.

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden.py

Writes, next to this script:
  kat_<name>.fa                 hand-written known-answer inputs
  kat_<name>.kmerGraph.txt      reference output, lines sorted by first token
  kat_<name>.nodes.txt          reference node lines, sorted by key
  cases.json                    every case: parameters, input hash, output
                                hashes, counts and the reference's totals
Synthetic cases are regenerated from their seeds by libswgsynth; only their
hashes are stored.
"""
from __future__ import annotations

import hashlib
import json
import shutil
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "swap-assembler_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402
import swapgb  # noqa: E402

from cases import KAT_CASES, SYNTH_CASES, synth_text  # noqa: E402


def sha(lines: list[str]) -> str:
    return hashlib.sha256(("\n".join(lines) + ("\n" if lines else "")).encode()).hexdigest()


def main() -> None:
    if not oracle.reference_available():
        sys.exit("oracle/_ref is not built (make -C oracle reference)")
    out = {"kat": [], "synth": []}
    tmp = Path(tempfile.mkdtemp(prefix="swg_golden_"))
    try:
        for case in KAT_CASES:
            fa = HERE / ("kat_%s.fa" % case["name"])
            fa.write_bytes(case["text"])
            res = oracle.run_reference(str(fa), case["k"], case["c"], str(tmp / case["name"]),
                                       timeout=60)
            (HERE / ("kat_%s.kmerGraph.txt" % case["name"])).write_text(
                "".join(l + "\n" for l in res["kmer_graph"]))
            (HERE / ("kat_%s.nodes.txt" % case["name"])).write_text(
                "".join(l + "\n" for l in res["nodes"]))
            out["kat"].append({
                "name": case["name"], "k": case["k"], "c": case["c"],
                "fasta_sha256": hashlib.sha256(case["text"]).hexdigest(),
                "kmer_graph_sha256": sha(res["kmer_graph"]), "nodes_sha256": sha(res["nodes"]),
                "n_nodes": len(res["nodes"]), "n_kmer_graph_lines": len(res["kmer_graph"]),
                "totals": res["totals"], "why": case["why"],
            })
            print("kat", case["name"], len(res["nodes"]), "nodes")
        for case in SYNTH_CASES:
            text = synth_text(case)
            fa = tmp / (case["name"] + ".fa")
            fa.write_bytes(text)
            res = oracle.run_reference(str(fa), case["k"], case["c"], str(tmp / case["name"]),
                                       timeout=3600)
            out["synth"].append({
                "name": case["name"], "k": case["k"], "c": case["c"], "params": case["params"],
                "fasta_sha256": hashlib.sha256(text).hexdigest(), "fasta_bytes": len(text),
                "kmer_graph_sha256": sha(res["kmer_graph"]), "nodes_sha256": sha(res["nodes"]),
                "n_nodes": len(res["nodes"]), "n_kmer_graph_lines": len(res["kmer_graph"]),
                "totals": res["totals"], "why": case["why"],
            })
            print("synth", case["name"], len(res["nodes"]), "nodes")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    (HERE / "cases.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
