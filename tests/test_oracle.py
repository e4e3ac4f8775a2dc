"""The CPU restatement (oracle/) pinned against the reference's own outputs.

Golden fixtures are the outputs of the reference itself (tests/golden/
make_golden.py); where the reference binaries are present (this container),
the restatement is also compared with a live reference run on fresh inputs.
"""
import random
import tempfile
from pathlib import Path

import numpy as np
import pytest

import oracle
from common import golden, kat_text, node_lines, sha_lines, sorted_lines, synth_case_text


def _oracle_files(text, k, c, tmp):
    g = oracle.build(text, k, c)
    g.write_kmer_graph(tmp / "kg.txt")
    g.write_node_lines(tmp / "nodes.txt")
    return g, sorted_lines(tmp / "kg.txt"), sorted_lines(tmp / "nodes.txt")


@pytest.mark.parametrize("case", [c["name"] for c in golden()["kat"]])
def test_oracle_matches_reference_kat(case, tmp_path):
    c = next(x for x in golden()["kat"] if x["name"] == case)
    g, kg, nodes = _oracle_files(kat_text(case), c["k"], c["c"], tmp_path)
    assert sha_lines(kg) == c["kmer_graph_sha256"]
    assert sha_lines(nodes) == c["nodes_sha256"]
    st = g.stats()
    if c["totals"]:
        assert st[0] == c["totals"]["recvNodeNum"]
        assert st[1] == c["totals"]["recvEdgeNum"]
        assert st[3] == c["totals"]["recvTipsNum"]
        assert st[4] == c["totals"]["recvBubbleNum"]


@pytest.mark.parametrize("case", [c["name"] for c in golden()["synth"]])
def test_oracle_matches_reference_synthetic(case, tmp_path):
    c = next(x for x in golden()["synth"] if x["name"] == case)
    text = synth_case_text(case)
    g, kg, nodes = _oracle_files(text, c["k"], c["c"], tmp_path)
    assert len(nodes) == c["n_nodes"]
    assert sha_lines(kg) == c["kmer_graph_sha256"]
    assert sha_lines(nodes) == c["nodes_sha256"]


def test_oracle_thread_count_invariant():
    text = synth_case_text("c2_small")
    k1, m1 = oracle.records(text, 31, 5, threads=1)
    k7, m7 = oracle.records(text, 31, 5, threads=7)
    assert np.array_equal(k1, k7) and np.array_equal(m1, m7)


def test_revcomp_and_neighbour_quirk():
    k = 21
    s = "ACGTTGCAAGGTCCATGACTA"
    enc = lambda t: int("".join("ACGT".index(ch).__str__() for ch in t), 4)
    rc = s[::-1].translate(str.maketrans("ACGT", "TGCA"))
    assert oracle.revcomp(enc(s), k) == enc(rc)
    # slot s of K: N = last k bases of K+base (s<4) or rc(K)+base (s>=4);
    # printed as N if N >= rc(N), else complement(N) with base s restored.
    key = max(enc(s), enc(rc))
    ks = s if enc(s) == key else rc
    for slot in range(8):
        d = ks if slot < 4 else ks[::-1].translate(str.maketrans("ACGT", "TGCA"))
        n = (d + "ACGT"[slot % 4])[1:]
        rn = n[::-1].translate(str.maketrans("ACGT", "TGCA"))
        if enc(n) >= enc(rn):
            want = enc(n)
        else:
            comp = list(n.translate(str.maketrans("ACGT", "TGCA")))
            comp[slot] = n[slot]
            want = enc("".join(comp))
        assert oracle.kmer_graph_neighbour(key, slot, k) == want


def test_parse_errors():
    with pytest.raises(oracle.OracleError) as e:
        oracle.parse(b">r1\nACGTACGTACGTACGTACGTAC", 19)
    assert e.value.code == -2
    with pytest.raises(oracle.OracleError) as e:
        oracle.parse(b"ACGT\n", 19)
    assert e.value.code == -1
    with pytest.raises(oracle.OracleError) as e:
        oracle.parse(b">r1\nACGT\x00ACGT\n", 19)
    assert e.value.code == -3


@pytest.mark.skipif(not oracle.reference_available(), reason="reference binaries not built here")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_oracle_matches_live_reference(seed, tmp_path):
    rng = random.Random(seed)
    k = rng.choice([19, 21, 23, 25, 27, 29, 31])
    c = rng.choice([0, 1, 2, 3, 5])
    g = "".join(rng.choice("ACGT") for _ in range(rng.randint(300, 3000)))
    reads = []
    for _ in range(rng.randint(50, 400)):
        L = rng.randint(10, 180)
        st = rng.randint(0, max(0, len(g) - L))
        r = g[st:st + L]
        if rng.random() < 0.5:
            r = r[::-1].translate(str.maketrans("ACGT", "TGCA"))
        r = "".join(ch if rng.random() > 0.02 else rng.choice("ACGTNacgtn") for ch in r)
        reads.append(r)
    text = "".join(">q%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode()
    fa = tmp_path / "in.fa"
    fa.write_bytes(text)
    ref = oracle.run_reference(str(fa), k, c, str(tmp_path / "ref"), timeout=120)
    keys, mult = oracle.records(text, k, c)
    assert node_lines(keys, mult) == ref["nodes"]
    og = oracle.build(text, k, c)
    og.write_kmer_graph(tmp_path / "kg.txt")
    assert sorted_lines(tmp_path / "kg.txt") == ref["kmer_graph"]
