"""The CPU restatement of the merge stage (oracle/merge_oracle.c) against the
reference: replaying the reference's own visiting order with its one-rank
message timing gives its -d output byte for byte, from the stored fixtures
(tests/golden/make_merge_golden.py) and, where the reference was compiled
here, live. Plus the properties the GPU merge relies on: the arc strings do
not depend on the visiting order, and a complete merge leaves no mergeable
node."""
import hashlib
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from cases import MERGE_CASES, SYNTH_CASES, case_text

GOLDEN = Path(__file__).resolve().parent / "golden"
MERGE_GOLDEN = json.loads((GOLDEN / "merge_cases.json").read_text())


def _lines(text: bytes) -> list[bytes]:
    return sorted(l for l in text.split(b"\n") if l)


def _arc_strings(text: bytes) -> dict[int, list[bytes]]:
    out = {}
    for line in text.split(b"\n"):
        if not line:
            continue
        head, rest = line.split(b" ", 1)
        fields = rest.split(b"#")[:8]
        out[int(head)] = [f.strip() for f in fields]
    return out


@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_merge_replays_reference_fixture(case):
    g = MERGE_GOLDEN[case["name"]]
    text = case_text(case)
    assert hashlib.sha256(text).hexdigest() == g["input_sha256"]
    keys, mult = oracle.records(text, case["k"], case["c"])
    assert keys.size == g["nodes"]
    order = np.load(GOLDEN / (case["name"] + ".order.npy")).astype(np.uint64)
    out = oracle.merge_text(keys, mult, case["k"], order=order, timing=oracle.MERGE_TIMING_REFERENCE)
    assert len(out) == g["merged_bytes"]
    assert hashlib.sha256(out).hexdigest() == g["merged_sha256"]


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not compiled here")
@pytest.mark.parametrize("case", [c for c in SYNTH_CASES if c["name"] in ("c1_small", "c3_small", "k25_c1")],
                         ids=lambda c: c["name"])
def test_merge_replays_live_reference(case, tmp_path):
    fa = tmp_path / "in.fa"
    fa.write_bytes(case_text(case))
    nodes, ref = oracle.run_reference_merge(str(fa), case["k"], case["c"], str(tmp_path / "o"))
    keys, mult = oracle.parse_node_lines(nodes)
    out = oracle.merge_text(keys, mult, case["k"], order=np.arange(keys.size),
                            timing=oracle.MERGE_TIMING_REFERENCE)
    assert out == ref


@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_arc_strings_do_not_depend_on_the_order(case):
    """Nodes with other than one arc per side are never merged and end up
    with the same arc strings whatever the order; only which node of an
    isolated cycle is left (and where its cycle string starts) depends on it."""
    keys, mult = oracle.records(case_text(case), case["k"], case["c"])
    ref_order = np.load(GOLDEN / (case["name"] + ".order.npy")).astype(np.uint64)
    rng = np.random.default_rng(7)
    texts = [oracle.merge_text(keys, mult, case["k"], order=o) for o in
             (None, ref_order, rng.permutation(keys.size).astype(np.uint64), np.arange(keys.size)[::-1].copy())]
    one_each = {int(key) for key, m in zip(keys, mult) if np.count_nonzero(m[:4]) == 1 and np.count_nonzero(m[4:]) == 1}
    arcs = [_arc_strings(t) for t in texts]
    ends = [{key: a for key, a in x.items() if key not in one_each} for x in arcs]
    for x, e in zip(arcs[1:], ends[1:]):
        assert e == ends[0]
        assert len(x) == len(arcs[0])
        assert sum(len(s) for v in x.values() for s in v) == sum(len(s) for v in arcs[0].values() for s in v)


@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_complete_merge_leaves_no_mergeable_node(case):
    k = case["k"]
    keys, mult = oracle.records(case_text(case), k, case["c"])
    out = oracle.merge_text(keys, mult, k)
    left = _arc_strings(out)
    codes = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}
    mask = (1 << (2 * k)) - 1
    for key, arcs in left.items():
        right = [s for s in range(4) if arcs[s]]
        lft = [s for s in range(4, 8) if arcs[s]]
        if len(right) != 1 or len(lft) != 1:
            continue
        # one arc per side: one of them must lead back to the node itself
        ends = []
        for s in (right[0], lft[0]):
            v = key if s < 4 else oracle.revcomp(key, k)
            for ch in arcs[s][-k:]:
                v = ((v << 2) | codes[ch]) & mask
            ends.append(max(v, oracle.revcomp(v, k)))
        assert key in ends, key


def test_reference_timing_keeps_what_a_complete_merge_removes():
    """At one rank the reference leaves nodes its pending messages kept
    locked and loses its last merge; the complete merge has fewer lines."""
    case = MERGE_CASES[0]
    keys, mult = oracle.records(case_text(case), case["k"], case["c"])
    order = np.load(GOLDEN / (case["name"] + ".order.npy")).astype(np.uint64)
    lazy = oracle.merge_text(keys, mult, case["k"], order=order, timing=oracle.MERGE_TIMING_REFERENCE)
    full = oracle.merge_text(keys, mult, case["k"], order=order)
    assert len(_lines(full)) < len(_lines(lazy))


def test_merge_tree_order_is_a_permutation():
    case = MERGE_CASES[2]
    keys, mult = oracle.records(case_text(case), case["k"], case["c"])
    order = oracle.merge_tree_order(keys, mult, case["k"])
    assert np.array_equal(np.sort(order), np.arange(keys.size, dtype=np.uint64))


def test_merge_of_nothing_is_one_newline():
    assert oracle.merge_text(np.zeros(0, np.uint64), np.zeros((0, 8), np.uint8), 21) == b"\n"


def _rc(s: str) -> str:
    return s[::-1].translate(str.maketrans("ACGT", "TGCA"))


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not compiled here")
@pytest.mark.parametrize("case", [MERGE_CASES[0], MERGE_CASES[1], MERGE_CASES[3]] +
                         [c for c in SYNTH_CASES if c["name"] == "c1_small"], ids=lambda c: c["name"])
def test_reference_contig_stage_reads_the_complete_merge(case, tmp_path):
    """Drop-in at the file seam: the reference's own contig stage, fed the
    complete merge (the GPU's output), prints the contigs of the reference's
    own run (noCEcontigs.fasta: arc strings only, no multiplicities) — except
    where the reference's lost last merge splits a contig in two: each
    contig only the reference prints is a piece of one only ours prints."""
    k, c = case["k"], case["c"]
    fa = tmp_path / "in.fa"
    fa.write_bytes(case_text(case))
    r = subprocess.run([str(oracle.REF_SWAP), "-k", str(k), "-c", str(c), "-i", str(fa), "-o",
                        str(tmp_path / "ref"), "-d"], stdout=subprocess.DEVNULL, timeout=600)
    assert r.returncode == 0
    theirs = set(oracle.contig_sequences(tmp_path / "ref" / "noCEcontigs.fasta"))
    keys, mult = oracle.records(case_text(case), k, c)
    merged = tmp_path / "contigGraph.txt"
    merged.write_bytes(oracle.merge_text(keys, mult, k))
    ours_list, _ = oracle.run_reference_contigs(str(merged), k, c, str(tmp_path / "ours"))
    ours = set(ours_list)
    only_ours, only_theirs = ours - theirs, theirs - ours
    assert len(only_ours) <= 1
    for piece in only_theirs:
        assert any(piece in s or _rc(piece) in s for s in only_ours)


# ---- masterTipsRemoval / masterLowCoverageEdgeRemoval on the complete merge

@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_prune_replays_reference_fixture(case):
    g = MERGE_GOLDEN[case["name"]]
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    order = np.load(GOLDEN / (case["name"] + ".prune_order.npy")).astype(np.uint64)
    tips, _ = oracle.prune_text(full, k, oracle.PRUNE_TIPS, order)
    assert len(tips) == g["tips_bytes"] and hashlib.sha256(tips).hexdigest() == g["tips_sha256"]
    low, _ = oracle.prune_text(full, k, oracle.PRUNE_TIPS | oracle.PRUNE_LOW_COVERAGE, order)
    assert len(low) == g["lowcov_bytes"] and hashlib.sha256(low).hexdigest() == g["lowcov_sha256"]


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not compiled here")
@pytest.mark.parametrize("case", [c for c in SYNTH_CASES if c["name"] in ("c1_small", "c3_small", "k25_c1")],
                         ids=lambda c: c["name"])
def test_prune_replays_live_reference(case, tmp_path):
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    mp = tmp_path / "merged.txt"
    mp.write_bytes(full)
    before, tips, low = oracle.run_reference_prune(str(mp), k, case["c"], str(tmp_path / "o"))
    assert oracle.prune_text(before, k, oracle.PRUNE_TIPS)[0] == tips
    assert oracle.prune_text(before, k, oracle.PRUNE_TIPS | oracle.PRUNE_LOW_COVERAGE)[0] == low


def test_prune_low_coverage_cuts_something():
    """At least one fixture exercises the low-coverage cut (not only tips)."""
    case = MERGE_CASES[1]
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    tips, n_tips = oracle.prune_text(full, k, oracle.PRUNE_TIPS)
    both, n_both = oracle.prune_text(full, k, oracle.PRUNE_TIPS | oracle.PRUNE_LOW_COVERAGE)
    assert n_tips > 0 and n_both > n_tips and both != tips


# ---- masterSimplifyNodeGraph over the lines left by a pass

@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_simplify_replays_reference_fixture(case):
    g = MERGE_GOLDEN[case["name"]]
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    tips, _ = oracle.prune_text(full, k, oracle.PRUNE_TIPS, oracle.tips_last_order(full, k))
    order = np.load(GOLDEN / (case["name"] + ".simplify_order.npy")).astype(np.uint64)
    out, _ = oracle.simplify_text(tips, k, order)
    assert len(out) == g["simplify_bytes"] and hashlib.sha256(out).hexdigest() == g["simplify_sha256"]


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not compiled here")
@pytest.mark.parametrize("case", [c for c in SYNTH_CASES if c["name"] in ("c1_small", "c3_small", "k25_c1")],
                         ids=lambda c: c["name"])
def test_simplify_replays_live_reference(case, tmp_path):
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    tips, _ = oracle.prune_text(full, k, oracle.PRUNE_TIPS)
    tp = tmp_path / "tips.txt"
    tp.write_bytes(tips)
    before, after = oracle.run_reference_simplify(str(tp), k, case["c"], str(tmp_path / "o"))
    assert oracle.simplify_text(before, k)[0] == after


def test_simplify_order_is_a_permutation_and_merges_as_many():
    case = MERGE_CASES[0]
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    tips, _ = oracle.prune_text(full, k, oracle.PRUNE_TIPS)
    order = oracle.lines_tree_order(tips, k)
    n = len([l for l in tips.split(b"\n") if l])
    assert np.array_equal(np.sort(order), np.arange(n, dtype=np.uint64))
    a, na = oracle.simplify_text(tips, k)
    b, nb = oracle.simplify_text(tips, k, order)
    assert na == nb > 0 and len(a) == len(b)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not compiled here")
@pytest.mark.parametrize("case", MERGE_CASES[:2] + [c for c in SYNTH_CASES if c["name"] == "c1_small"],
                         ids=lambda c: c["name"])
def test_contigs_of_the_complete_merge_match_the_reference_writer(case, tmp_path):
    """printContigs restated (oracle.contigs_of_lines) equals the reference's
    own noCEcontigs.fasta on the same merged graph (its contig stage run on
    the complete merge; its masterSimplifyNodeGraph finds nothing to merge)."""
    k = case["k"]
    full = oracle.merge_text(*oracle.records(case_text(case), k, case["c"]), k)
    mp = tmp_path / "merged.txt"
    mp.write_bytes(full)
    theirs, _ = oracle.run_reference_contigs(str(mp), k, case["c"], str(tmp_path / "o"))
    assert oracle.contigs_of_lines(full, k) == theirs
