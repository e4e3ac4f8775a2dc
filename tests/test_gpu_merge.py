"""GPU merge of semi-extended k-molecules (swg_graph_merge) against the CPU
restatement run in the same visiting order with every message applied at
once (oracle/merge_oracle.c). The lines must be identical (the device writes
them in key order, the restatement in visiting order, so lines are compared
as sorted sets), and the file sizes equal."""
import subprocess
from pathlib import Path

import pytest

import oracle
import swapgb
from cases import MERGE_CASES, SYNTH_CASES, case_text

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
SWAP = ROOT / "swap-assembler_gb300" / "bin" / "swap"


def _lines(text: bytes) -> list[bytes]:
    return sorted(l for l in text.split(b"\n") if l)


def _gpu_merge(text: bytes, k: int, c: int, algorithm: int = swapgb.ALGO_DEFAULT) -> tuple[bytes, dict]:
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c, algorithm=algorithm), text)
    g.merge()
    return g.merged_text(), g.merge_info()


def _check(text: bytes, k: int, c: int, algorithm: int = swapgb.ALGO_DEFAULT) -> dict:
    got, info = _gpu_merge(text, k, c, algorithm)
    keys, mult = oracle.records(text, k, c)
    want = oracle.merge_text(keys, mult, k)
    assert len(got) == len(want) == info["text_bytes"]
    assert got.endswith(b"\n")
    gl, wl = _lines(got), _lines(want)
    assert len(gl) == len(wl) == info["nodes"]
    assert gl == wl
    firsts = [int(l.split(b" ", 1)[0]) for l in got.split(b"\n") if l]
    assert firsts == sorted(firsts)  # key order
    return info


@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_merge_matches_oracle(case):
    info = _check(case_text(case), case["k"], case["c"])
    if case["name"] == "merge_cycles_k23":
        assert info["cycles"] >= 3


@pytest.mark.parametrize("case", [c for c in SYNTH_CASES if c["name"] != "c1_full"], ids=lambda c: c["name"])
def test_merge_matches_oracle_synthetic(case):
    _check(case_text(case), case["k"], case["c"])


def test_merge_same_for_both_builds():
    case = MERGE_CASES[0]
    text = case_text(case)
    a, _ = _gpu_merge(text, case["k"], case["c"], swapgb.ALGO_BUCKETED)
    b, _ = _gpu_merge(text, case["k"], case["c"], swapgb.ALGO_DIRECT)
    assert a == b


def test_merge_full_size_workload():
    """The 1 Mbp, 300k-read workload: about a million k-molecules."""
    case = next(c for c in SYNTH_CASES if c["name"] == "c1_full")
    info = _check(case_text(case), case["k"], case["c"])
    assert info["chains"] > 0


def test_merge_long_chains():
    """An error-free 400 kbp genome at high cutoff: few, very long chains
    (the ruling-set walks and the deep reduction levels)."""
    text = swapgb.synth_fasta(seed=77, genome_len=400_000, n_reads=200_000, read_len=100, sub_rate=0.0)
    info = _check(text, 31, 3)
    assert info["nodes"] < 1000


def test_merge_cycles_of_every_size():
    """Isolated cycles of length 1 (a node whose arcs lead to itself), 2, 3,
    5 and a circular genome."""
    import random
    rng = random.Random(5)
    g = "".join(rng.choice("ACGT") for _ in range(3000))
    reads = [g[i:i + 100] if i + 100 <= 3000 else g[i:] + g[:i + 100 - 3000] for i in range(0, 3000, 7)]
    units = ["A", "AC", "ACG", "ACGTT", "AACCGGTTAC"]
    reads += [u * (120 // len(u)) for u in units for _ in range(4)]
    text = "".join(">r%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode()
    for k in (19, 25, 31):
        _check(text, k, 2)


def test_merge_empty_graph():
    text = swapgb.synth_fasta(seed=8, genome_len=5000, n_reads=100, read_len=100)
    got, info = _gpu_merge(text, 21, 255)
    assert got == b"\n" and info["nodes"] == 0


def test_merge_file_and_states(tmp_path):
    case = MERGE_CASES[1]
    g = swapgb.Graph()
    with pytest.raises(swapgb.SwgError):
        g.merge()  # nothing built
    g.build_fasta(swapgb.Opts(k=case["k"], cutoff=case["c"]), case_text(case))
    with pytest.raises(swapgb.SwgError):
        g.merged_text()  # not merged yet
    g.merge()
    p = tmp_path / "contigGraph.txt"
    g.write_merged(str(p))
    assert p.read_bytes() == g.merged_text()
    g.build_fasta(swapgb.Opts(k=case["k"], cutoff=case["c"]), case_text(case))
    with pytest.raises(swapgb.SwgError):
        g.merge_info()  # a new build drops the merged graph
    r = swapgb.reads_from_fasta(case_text(case), case["k"])
    g.build_batch(swapgb.Opts(), [(r, case["k"], case["c"])])
    with pytest.raises(swapgb.SwgError):
        g.merge()  # batched results are per sample
    g.build_fasta(swapgb.Opts(k=20, cutoff=2), case_text(case))
    with pytest.raises(swapgb.SwgError):
        g.merge()  # even k


def test_cli_writes_contig_graph(tmp_path):
    case = MERGE_CASES[0]
    fa = tmp_path / "in.fa"
    fa.write_bytes(case_text(case))
    out = tmp_path / "o"
    r = subprocess.run([str(SWAP), "-k", str(case["k"]), "-c", str(case["c"]), "-i", str(fa), "-o", str(out),
                        "-d"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    got = (out / "contigGraph.txt").read_bytes()
    keys, mult = oracle.records(case_text(case), case["k"], case["c"])
    assert _lines(got) == _lines(oracle.merge_text(keys, mult, case["k"]))
    assert "Simplify DistGraph" in (out / "logtime.txt").read_text()
    assert oracle.contig_sequences(out / "noCEcontigs.fasta") == oracle.contigs_of_lines(got, case["k"])
    # with -s the reference stops after kmerGraph.txt: no merge
    out2 = tmp_path / "o2"
    r = subprocess.run([str(SWAP), "-k", str(case["k"]), "-c", str(case["c"]), "-i", str(fa), "-o", str(out2),
                        "-d", "-s"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert (out2 / "kmerGraph.txt").exists() and not (out2 / "contigGraph.txt").exists()


PRUNE_CASES = MERGE_CASES + [c for c in SYNTH_CASES if c["name"] in ("c1_small", "c3_small", "k25_c1")]


@pytest.mark.parametrize("case", PRUNE_CASES, ids=lambda c: c["name"])
def test_tip_and_low_coverage_passes_match_oracle(case):
    """swg_graph_remove_tips / _low_coverage on the merged graph against the
    restatement of masterTipsRemoval / masterLowCoverageEdgeRemoval visiting
    every non-tip first and then the tips in key order."""
    k, c = case["k"], case["c"]
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), case_text(case))
    g.merge()
    before = g.merged_text()
    order = oracle.tips_last_order(before, k)
    removed = g.remove_tips()
    tips = g.merged_text()
    want, n = oracle.prune_text(before, k, oracle.PRUNE_TIPS, order)
    assert removed == n
    assert _lines(tips) == _lines(want) and len(tips) == len(want)
    assert g.merge_info()["nodes"] == len(_lines(tips))
    cut = g.remove_low_coverage()
    low = g.merged_text()
    want2, n2 = oracle.prune_text(before, k, oracle.PRUNE_TIPS | oracle.PRUNE_LOW_COVERAGE, order)
    assert cut == n2 - n
    assert _lines(low) == _lines(want2) and len(low) == len(want2)
    firsts = [int(l.split(b" ", 1)[0]) for l in low.split(b"\n") if l]
    assert firsts == sorted(firsts)


def test_prune_states_and_repeat():
    """The passes need a merged graph; a second tip pass removes the tips the
    first one left (nodes whose other arcs went with the first tips), as the
    restatement's second pass does."""
    k = 21
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=1), case_text(MERGE_CASES[0]))
    with pytest.raises(swapgb.SwgError):
        g.remove_tips()  # not merged
    g.merge()
    before = g.merged_text()
    assert g.remove_tips() > 0
    once = g.merged_text()
    want1, _ = oracle.prune_text(before, k, oracle.PRUNE_TIPS, oracle.tips_last_order(before, k))
    assert _lines(once) == _lines(want1)
    second = g.remove_tips()
    want2, n2 = oracle.prune_text(once, k, oracle.PRUNE_TIPS, oracle.tips_last_order(once, k))
    assert second == n2 and _lines(g.merged_text()) == _lines(want2)


@pytest.mark.parametrize("case", PRUNE_CASES, ids=lambda c: c["name"])
def test_simplify_after_the_passes_matches_oracle(case):
    """The reference's sequence tip pass -> masterSimplifyNodeGraph ->
    low-coverage pass -> masterSimplifyNodeGraph on the merged graph: each
    GPU step equals the restatement (the simplify in the GPU's visiting order
    of the lines, oracle_lines_tree_order)."""
    k, c = case["k"], case["c"]
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), case_text(case))
    g.merge()
    g.remove_tips()
    tips = g.merged_text()
    merged = g.simplify()
    want, n = oracle.simplify_text(tips, k, oracle.lines_tree_order(tips, k))
    got = g.merged_text()
    assert merged == n
    assert _lines(got) == _lines(want) and len(got) == len(want)
    assert g.merge_info()["nodes"] == len(_lines(got))
    g.remove_low_coverage()
    low = g.merged_text()
    g.simplify()
    want2, _ = oracle.simplify_text(low, k, oracle.lines_tree_order(low, k))
    assert _lines(g.merged_text()) == _lines(want2)
    # nothing left to merge
    assert g.simplify() == 0


def test_simplify_cycles():
    """A cycle left when a tip that held its only branch goes: cut at its
    largest key, as the restatement's visiting order does."""
    import random
    rng = random.Random(9)
    g0 = "".join(rng.choice("ACGT") for _ in range(2000))
    reads = [g0[i:i + 100] if i + 100 <= 2000 else g0[i:] + g0[:i + 100 - 2000] for i in range(0, 2000, 5)]
    # three short spurs off the circle: tips once merged; without them the
    # three branch nodes form a cycle of one-arc-per-side nodes
    for at in (300, 900, 1500):
        spur = g0[at:at + 30] + "".join(rng.choice("ACGT") for _ in range(5))
        reads += [spur] * 6
    text = "".join(">r%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode()
    for k in (21, 25):
        g = swapgb.Graph()
        g.build_fasta(swapgb.Opts(k=k, cutoff=2), text)
        g.merge()
        g.remove_tips()
        tips = g.merged_text()
        assert g.simplify() == 2
        want, _ = oracle.simplify_text(tips, k, oracle.lines_tree_order(tips, k))
        assert _lines(g.merged_text()) == _lines(want) and len(_lines(want)) == 1


@pytest.mark.parametrize("case", PRUNE_CASES[:4], ids=lambda c: c["name"])
def test_contigs_match_oracle(case, tmp_path):
    """swg_graph_write_contigs (printContigs) on the merged graph, and again
    after the tip pass and re-merge, against the restatement on the same
    lines; the file holds exactly the '>proc0: ' lines."""
    k, c = case["k"], case["c"]
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), case_text(case))
    g.merge()
    for step in range(2):
        p = tmp_path / ("contigs%d.fasta" % step)
        n = g.write_contigs(str(p))
        body = p.read_bytes()
        assert body.count(b"\n") == n and all(l.startswith(b">proc0: ") for l in body.split(b"\n") if l)
        assert oracle.contig_sequences(p) == oracle.contigs_of_lines(g.merged_text(), k)
        g.remove_tips()
        g.simplify()


# ---- merge in a given visiting order (swg_graph_merge_in_order) ----------
GOLDEN = ROOT / "tests" / "golden"


def _ordered(text: bytes, k: int, c: int, order):
    """GPU merge visiting the nodes in `order` (indices of the key-sorted
    k-molecules) and the restatement in the same order, every message
    applied as it is sent (MERGE_TIMING_IMMEDIATE)."""
    import numpy as np
    keys, mult = oracle.records(text, k, c)
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), text)
    g.merge_in_order(keys[np.asarray(order, dtype=np.int64)])
    want = oracle.merge_text(keys, mult, k, order=order, timing=oracle.MERGE_TIMING_IMMEDIATE)
    return g.merged_text(), want, g.merge_info()


@pytest.mark.parametrize("case", MERGE_CASES, ids=lambda c: c["name"])
def test_merge_in_the_reference_order(case):
    """The reference's own visiting order of each merge fixture (its node
    map's iteration order, stored by tests/golden/make_merge_golden.py from
    the reference's run): the GPU merge equals the restatement replaying that
    order line for line, multiplicities included (graph.cpp:1392-1566,
    averaging at 1322-1324)."""
    import numpy as np
    order = np.load(GOLDEN / (case["name"] + ".order.npy")).astype(np.uint64)
    got, want, info = _ordered(case_text(case), case["k"], case["c"], order)
    assert len(got) == len(want) == info["text_bytes"]
    assert _lines(got) == _lines(want)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_merge_in_random_orders(seed):
    """Random visiting orders on a graph of a few long chains and on the
    1 Mbp workload's graph (deep and shallow merge trees, cycles)."""
    import numpy as np
    for text, k, c in ((swapgb.synth_fasta(seed=77, genome_len=100_000, n_reads=50_000, read_len=100,
                                           sub_rate=0.0), 31, 3),
                       (case_text(next(x for x in SYNTH_CASES if x["name"] == "c1_small")), 21, 2)):
        n = oracle.records(text, k, c)[0].size
        order = np.random.default_rng(seed).permutation(n).astype(np.uint64)
        got, want, _ = _ordered(text, k, c, order)
        assert _lines(got) == _lines(want)


def test_merge_in_the_fixed_order_equals_merge():
    """Given the fixed tree order itself, the ordered merge reproduces
    swg_graph_merge byte for byte."""
    case = MERGE_CASES[2]
    text, k, c = case_text(case), case["k"], case["c"]
    keys, mult = oracle.records(text, k, c)
    order = oracle.merge_tree_order(keys, mult, k)
    a, _ = _gpu_merge(text, k, c)
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), text)
    g.merge_in_order(keys[order.astype("int64")])
    assert g.merged_text() == a


def test_merge_in_order_rejects_bad_orders():
    import numpy as np
    case = MERGE_CASES[1]
    text, k, c = case_text(case), case["k"], case["c"]
    keys, _ = oracle.records(text, k, c)
    g = swapgb.Graph()
    g.build_fasta(swapgb.Opts(k=k, cutoff=c), text)
    bad = [keys[:-1], np.concatenate([keys[:-1], keys[:1]]), np.concatenate([keys[:-1], [np.uint64(1)]])]
    for order in bad:  # a key missing, a key twice, a key the graph does not hold
        with pytest.raises(swapgb.SwgError) as e:
            g.merge_in_order(order)
        assert e.value.status == 1
    g.merge_in_order(keys[::-1].copy())  # and a good one still works on the same handle
