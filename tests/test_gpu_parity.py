"""GPU parity: the sm_103a build through the C ABI against the reference's
own outputs (golden fixtures) and the CPU restatement. Integer work, so the
bar is bit-exact equality of every key and every multiplicity."""
import numpy as np
import pytest

import oracle
import swapgb
from common import golden, kat, kat_text, sha_lines, sorted_lines, synth_case, synth_case_text

pytestmark = pytest.mark.gpu


def gpu_build(text: bytes, k: int, c: int, **kw) -> swapgb.Graph:
    reads = swapgb.reads_from_fasta(text, k)
    g = swapgb.Graph()
    g.build_reads(swapgb.Opts(k=k, cutoff=c, **kw), reads)
    return g


def assert_same_records(g: swapgb.Graph, text: bytes, k: int, c: int) -> None:
    keys, mult = g.copy_out(sorted=True)
    okeys, omult = oracle.records(text, k, c)
    assert keys.size == okeys.size, (keys.size, okeys.size)
    assert np.array_equal(keys, okeys)
    bad = np.nonzero((mult != omult).any(axis=1))[0]
    assert bad.size == 0, "first mismatch key=%d gpu=%s oracle=%s" % (
        keys[bad[0]], mult[bad[0]].tolist(), omult[bad[0]].tolist())


# (algorithm, read order): direct in input order (the default), direct in
# minimizer order, partitioned, bucketed
ALGOS = [pytest.param(dict(algorithm=swapgb.ALGO_DIRECT), id="direct"),
         pytest.param(dict(algorithm=swapgb.ALGO_DIRECT, read_order=swapgb.ORDER_MINIMIZER),
                      id="direct-minimizer-order"),
         pytest.param(dict(algorithm=swapgb.ALGO_PARTITIONED), id="partitioned"),
         pytest.param(dict(algorithm=swapgb.ALGO_BUCKETED), id="bucketed")]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("case", [c["name"] for c in golden()["kat"]])
def test_kat_matches_reference(case, algo, tmp_path):
    c = kat(case)
    g = gpu_build(kat_text(case), c["k"], c["c"], **algo)
    assert g.info()["algorithm"] == algo["algorithm"]
    g.write_kmer_graph(tmp_path / "kg.txt")
    g.write_node_lines(tmp_path / "nodes.txt")
    assert sha_lines(sorted_lines(tmp_path / "kg.txt")) == c["kmer_graph_sha256"]
    assert sha_lines(sorted_lines(tmp_path / "nodes.txt")) == c["nodes_sha256"]
    assert g.size() == c["n_nodes"]
    if c["totals"]:
        st = g.stats()
        assert st[0] == c["totals"]["recvNodeNum"] and st[1] == c["totals"]["recvEdgeNum"]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("case", [c["name"] for c in golden()["synth"]])
def test_synthetic_matches_reference(case, algo, tmp_path):
    c = synth_case(case)
    text = synth_case_text(case)
    g = gpu_build(text, c["k"], c["c"], **algo)
    assert g.size() == c["n_nodes"]
    g.write_node_lines(tmp_path / "nodes.txt")
    assert sha_lines(sorted_lines(tmp_path / "nodes.txt")) == c["nodes_sha256"]
    g.write_kmer_graph(tmp_path / "kg.txt")
    assert sha_lines(sorted_lines(tmp_path / "kg.txt")) == c["kmer_graph_sha256"]


@pytest.mark.parametrize("k,c", [(19, 0), (21, 1), (23, 2), (27, 3), (29, 4), (31, 5), (31, -3),
                                 (9, 2), (15, 1), (20, 2), (1, 1), (2, 0)])
@pytest.mark.parametrize("algo", ALGOS)
def test_k_and_cutoff_sweep(k, c, algo):
    text = synth_case_text("c2_small")
    g = gpu_build(text, k, c, **algo)
    assert_same_records(g, text, k, c)


@pytest.mark.parametrize("algo", ALGOS)
def test_repeats_and_tandems(algo):
    text = swapgb.synth_fasta(seed=21, genome_len=300000, repeat_frac=0.05, tandem_frac=0.02,
                              n_reads=60000, read_len=150, sub_rate=0.005)
    g = gpu_build(text, 31, 3, **algo)
    assert_same_records(g, text, 31, 3)


@pytest.mark.parametrize("algo", ALGOS)
def test_hot_keys_saturate(algo):
    # one k-mer hit millions of times inside single warps: poly-A and short
    # tandem units; counts must saturate at exactly 255
    reads = ["A" * 250, "AC" * 125, "ACG" * 83, "T" * 200, "ACGTT" * 50] * 4000
    text = "".join(">h%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode()
    for c in (0, 2, 255):
        g = gpu_build(text, 21, c, **algo)
        assert_same_records(g, text, 21, c)
        _, mult = g.copy_out()
        assert mult.max() == 255


def test_partitioned_multi_wave_and_larger_input():
    # enough occurrences for more partitions than one wave holds
    text = swapgb.synth_fasta(seed=23, genome_len=2_000_000, n_reads=1_000_000, read_len=100,
                              sub_rate=0.01, indel_rate=0.001)
    g = gpu_build(text, 31, 5, algorithm=swapgb.ALGO_PARTITIONED)
    info = g.info()
    assert info["waves"] > 1 and info["partitions"] >= 256
    assert_same_records(g, text, 31, 5)
    assert info["occurrences"] == 70_000_000


def test_table_full_retry():
    # a sizing hint far too small forces the device-side full detection and
    # the host's rebuild with a larger table (direct algorithm)
    text = synth_case_text("c1_small")
    g = gpu_build(text, 21, 2, expected_distinct=10, algorithm=swapgb.ALGO_DIRECT)
    assert_same_records(g, text, 21, 2)
    assert g.info()["retries"] >= 1


@pytest.mark.parametrize("algo", ALGOS)
def test_high_load_factor(algo):
    text = synth_case_text("c2_small")
    g = gpu_build(text, 31, 5, load_factor=0.9, **algo)
    assert_same_records(g, text, 31, 5)


@pytest.mark.parametrize("algo", ALGOS)
def test_empty_and_short_inputs(algo):
    text = b">a\nACGT\n>b\nAC\n"  # every read shorter than k
    g = gpu_build(text, 19, 0, **algo)
    assert g.size() == 0 and g.distinct() == 0
    text = b">a\nACGTACGTACGTACGTACGTA\n"  # L == k: one key, all-zero mask, dropped
    g = gpu_build(text, 21, 0, **algo)
    assert g.size() == 0 and g.distinct() == 1


def test_device_input_path_and_handle_reuse():
    import torch
    text1 = synth_case_text("c2_small")
    text2 = synth_case_text("c4_ragged")
    g = swapgb.Graph()
    for text, k, c, algo, order in ((text1, 31, 5, 2, 0), (text2, 27, 3, 1, 1),
                                    (text1, 31, 5, 1, 0), (text2, 27, 3, 2, 0),
                                    (text1, 31, 5, 1, 1)):
        r = swapgb.reads_from_fasta(text, k)
        p = torch.from_numpy(r.packed.view(np.int32).copy()).cuda()
        o = torch.from_numpy(r.off.view(np.int64).copy()).cuda()
        ln = torch.from_numpy(r.len.view(np.int32).copy()).cuda()
        torch.cuda.synchronize()
        g.build_device(swapgb.Opts(k=k, cutoff=c, algorithm=algo, read_order=order),
                       p.data_ptr(), p.numel(), o.data_ptr(),
                       ln.data_ptr(), o.numel())
        assert_same_records(g, text, k, c)
        ms, launches = g.timings()
        assert launches >= 6 and ms[4] > 0


def test_unsorted_copy_is_a_permutation():
    text = synth_case_text("k25_c1")
    g = gpu_build(text, 25, 1)
    k1, m1 = g.copy_out(sorted=False)
    order = np.argsort(k1, kind="stable")
    k2, m2 = g.copy_out(sorted=True)
    assert np.array_equal(k1[order], k2) and np.array_equal(m1[order], m2)


def test_build_fasta_entry_point():
    text = kat_text("orient_k19")
    g = swapgb.build_fasta(swapgb.Opts(k=19, cutoff=1), text)
    assert_same_records(g, text, 19, 1)


@pytest.mark.parametrize("case", ["orient_k19", "crlf_k19", "multiline_k19", "saturate_k21"])
def test_build_fasta_file_entry_point(case, tmp_path):
    c = kat(case)
    fa = tmp_path / "in.fa"
    fa.write_bytes(kat_text(case))
    g = swapgb.Graph()
    for _ in range(2):  # the second call reuses the handle's pinned buffer
        g.build_fasta_file(swapgb.Opts(k=c["k"], cutoff=c["c"]), fa)
        g.write_kmer_graph(tmp_path / "kg.txt")
        g.write_node_lines(tmp_path / "nodes.txt")
        assert sha_lines(sorted_lines(tmp_path / "kg.txt")) == c["kmer_graph_sha256"]
        assert sha_lines(sorted_lines(tmp_path / "nodes.txt")) == c["nodes_sha256"]
    with pytest.raises(swapgb.SwgError) as e:
        g.build_fasta_file(swapgb.Opts(k=c["k"], cutoff=c["c"]), tmp_path / "missing.fa")
    assert e.value.status == 9  # SWG_ERR_IO


def test_cli_matches_reference(tmp_path):
    import subprocess
    c = kat("orient_k31_c3")
    fa = tmp_path / "in.fa"
    fa.write_bytes(kat_text("orient_k31_c3"))
    out = tmp_path / "out"
    r = subprocess.run([str(swapgb.SWAP_BIN), "-k", "31", "-c", "3", "-i", str(fa), "-o", str(out),
                        "-s"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    assert sha_lines(sorted_lines(out / "kmerGraph.txt")) == c["kmer_graph_sha256"]
    assert sha_lines(sorted_lines(out / "nodes.txt")) == c["nodes_sha256"]
    assert "recvNodeNum = %d" % c["totals"]["recvNodeNum"] in r.stdout


@pytest.mark.parametrize("case", [c["name"] for c in golden()["kat"]])
def test_device_framing_matches_reference(case, tmp_path):
    c = kat(case)
    g = swapgb.Graph().build_fasta(swapgb.Opts(k=c["k"], cutoff=c["c"]), kat_text(case))
    g.write_kmer_graph(tmp_path / "kg.txt")
    g.write_node_lines(tmp_path / "nodes.txt")
    assert sha_lines(sorted_lines(tmp_path / "kg.txt")) == c["kmer_graph_sha256"]
    assert sha_lines(sorted_lines(tmp_path / "nodes.txt")) == c["nodes_sha256"]


@pytest.mark.parametrize("case", ["c1_full", "c4_ragged", "c3_small"])
def test_device_framing_synthetic(case):
    c = synth_case(case)
    text = synth_case_text(case)
    g = swapgb.Graph().build_fasta(swapgb.Opts(k=c["k"], cutoff=c["c"]), text)
    assert g.size() == c["n_nodes"]
    assert_same_records(g, text, c["k"], c["c"])


def test_device_framing_odd_inputs():
    # leading bytes before the first '>', records shorter than k, CRLF
    text = b"junk\n\n>a\nACGTACGTACGTACGTACGTACGTTTGCA\r\n>b\nAC\n>c\n" + b"ACGT" * 40 + b"\n"
    g = swapgb.Graph().build_fasta(swapgb.Opts(k=19, cutoff=0), text)
    k1, m1 = g.copy_out()
    g2 = gpu_build(text, 19, 0)
    k2, m2 = g2.copy_out()
    assert np.array_equal(k1, k2) and np.array_equal(m1, m2)
    for bad in (b">r1\nACGTACGTACGTACGTACGTAC", b">r1\nACGTACGTACGTACGTACGTAC\n>r2\n",
                b"ACGTACGTACGTACGTACGTAC\n", b">r1\nACGTACGT\x00ACGTACGTACGTAC\n"):
        with pytest.raises(swapgb.SwgError) as e:
            swapgb.Graph().build_fasta(swapgb.Opts(k=19, cutoff=0), bad)
        assert e.value.status == 1


def test_autotune_then_build(tmp_path):
    import torch
    text = synth_case_text("c2_small")
    r = swapgb.reads_from_fasta(text, 31)
    p = torch.from_numpy(r.packed.view(np.int32).copy()).cuda()
    o = torch.from_numpy(r.off.view(np.int64).copy()).cuda()
    ln = torch.from_numpy(r.len.view(np.int32).copy()).cuda()
    cache = tmp_path / "tune.jsonl"
    best = swapgb.autotune(swapgb.Opts(k=31, cutoff=5), p.data_ptr(), p.numel(), o.data_ptr(),
                           ln.data_ptr(), o.numel(), 100, cache)
    assert best["algorithm"] in (1, 2, 3) and 0.5 <= best["load_factor"] <= 0.8 and best["ms"] > 0
    assert best["bucket_records"] in (0, 2048, 4096, 8192) and best["part_bits"] == 0
    assert best["scatter_shape"] in (0, 1, 2)
    opts = swapgb.Opts(k=31, cutoff=5)
    assert swapgb.autotune_apply(cache, 31, 100, opts)
    assert (opts.bucket_records, opts.part_bits, opts.scatter_shape) == (
        best["bucket_records"], best["part_bits"], best["scatter_shape"])
    g = swapgb.Graph().build_reads(opts, r)
    assert_same_records(g, text, 31, 5)


@pytest.mark.parametrize("knobs", [dict(bucket_records=2048), dict(bucket_records=8192, part_bits=9),
                                   dict(part_bits=10, scatter_shape=1), dict(scatter_shape=2),
                                   dict(scatter_shape=3, bucket_records=1024), dict(scatter_shape=4),
                                   dict(scatter_shape=4, part_bits=9)])
def test_bucketed_knobs_give_the_same_graph(knobs):
    """Every bucket size, partition count and scatter shape the autotuner may
    pick builds the same graph."""
    text = synth_case_text("c2_small")
    g = swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=5, algorithm=swapgb.ALGO_BUCKETED, **knobs),
                                   swapgb.reads_from_fasta(text, 31))
    assert g.info()["algorithm"] == swapgb.ALGO_BUCKETED
    assert_same_records(g, text, 31, 5)
    with pytest.raises(swapgb.SwgError):  # out of range
        swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=5, part_bits=11), swapgb.reads_from_fasta(text, 31))


@pytest.mark.parametrize("mode", ["auto", "0", "2"])
@pytest.mark.parametrize("records", [2048, 8192])
def test_tier1_table_choice(mode, records, monkeypatch):
    """The first counting pass takes 2048-entry tables when the plan's buckets
    average at most 3072 records (SWG_BUCKET_SMALL=0 / 2 force 4096 / 2048),
    and either gives the same graph, with hot repeats overflowing to the later tiers."""
    if mode != "auto":
        monkeypatch.setenv("SWG_BUCKET_SMALL", mode)
    text = synth_case_text("c2_small")
    hot = "".join(">h%d\n%s\n" % (i, r) for i, r in enumerate(["ACGTTGCA" * 20] * 3000)).encode()
    text = text + hot
    g = swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=5, algorithm=swapgb.ALGO_BUCKETED,
                                               bucket_records=records), swapgb.reads_from_fasta(text, 31))
    info = g.info()
    small = info["occurrences"] <= 3072 * info["table_entries"]
    want = {"auto": 2048 if small else 4096, "0": 4096, "2": 2048}[mode]
    assert info["bucket_table"] == want, info
    assert_same_records(g, text, 31, 5)


def test_bucketed_large_input_and_hot_buckets():
    text = swapgb.synth_fasta(seed=23, genome_len=2_000_000, n_reads=1_000_000, read_len=100,
                              sub_rate=0.01, indel_rate=0.001)
    g = gpu_build(text, 31, 5, algorithm=swapgb.ALGO_BUCKETED)
    assert_same_records(g, text, 31, 5)
    # one k-mer repeated far more often than a shared-memory bucket holds
    reads = ["A" * 250, "AC" * 125] * 30000 + ["ACGTTGCA" * 20] * 500
    text = "".join(">h%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode()
    g = gpu_build(text, 21, 2, algorithm=swapgb.ALGO_BUCKETED)
    info = g.info()
    assert info["waves"] >= 1, info  # global-memory path taken
    assert_same_records(g, text, 21, 2)


def test_bucketed_sampling_miss_recounts():
    """Partitions and buckets are sized from every 16th batch of 256 reads; a
    hot key that lives only in unsampled reads overflows its region, and the
    build reruns with exact counts."""
    text = swapgb.synth_fasta(seed=41, genome_len=12_000_000, n_reads=600_000, read_len=150,
                              sub_rate=0.005)  # 72M occurrences: the sampled sizing
    lines = text.split(b"\n")
    hot = b"".join(b">hot%d\n%s\n" % (i, b"A" * 250) for i in range(250))
    # reads 300..549: batches 1-2 of 256 reads, which the sample skips
    text = b"\n".join(lines[:600]) + b"\n" + hot + b"\n".join(lines[600:])
    g = gpu_build(text, 31, 2, algorithm=swapgb.ALGO_BUCKETED)
    info = g.info()
    assert info["estimate"] == 1.0, info  # the exact recount ran
    assert_same_records(g, text, 31, 2)


def test_bucketed_overflow_tiers(monkeypatch):
    """Buckets of nearly distinct k-molecules larger than the tier-1 table:
    recounted in the tier-2 table; larger still: the global-memory path."""
    monkeypatch.setenv("SWG_BUCKET_RECORDS", "1000000")  # one bucket per partition
    # 0.1x coverage of a random genome: almost every k-molecule is distinct,
    # ~5.8K per bucket (tier-1 tables hold 4096)
    text = swapgb.synth_fasta(seed=29, genome_len=20_000_000, n_reads=20_000, read_len=100,
                              sub_rate=0.0, indel_rate=0.0)
    g = gpu_build(text, 27, 0, algorithm=swapgb.ALGO_BUCKETED)
    info = g.info()
    assert info["slots"] == 1 and info["retries"] >= 1, info
    assert_same_records(g, text, 27, 0)
    # ~11.6K distinct per bucket: beyond the tier-2 tables (8192)
    text = swapgb.synth_fasta(seed=31, genome_len=40_000_000, n_reads=40_000, read_len=100,
                              sub_rate=0.0, indel_rate=0.0)
    g = gpu_build(text, 27, 1, algorithm=swapgb.ALGO_BUCKETED)
    info = g.info()
    assert info["waves"] >= 1, info
    assert_same_records(g, text, 27, 1)


@pytest.mark.parametrize("k,c", [(9, 2), (20, 0), (21, 2), (31, 3)])
def test_device_text_equals_host_writers(k, c, tmp_path):
    """kmerGraph.txt and the node lines formatted on the device are byte-for-
    byte the host writers' output for the same records (odd and even k: the
    neighbour-id quirk depends on k's parity; c=0 keeps every arc)."""
    text = swapgb.synth_fasta(seed=61 + k, genome_len=200_000, n_reads=40_000, read_len=100,
                              sub_rate=0.01, repeat_frac=0.05, tandem_frac=0.02)
    g = gpu_build(text, k, c)
    g.write_kmer_graph(tmp_path / "dev_kmerGraph.txt")
    g.write_node_lines(tmp_path / "dev_nodes.txt")
    keys, mult = g.copy_out(sorted=False)
    swapgb.records_write_kmer_graph(keys, mult, k, tmp_path / "host_kmerGraph.txt")
    swapgb.records_write_node_lines(keys, mult, tmp_path / "host_nodes.txt")
    assert (tmp_path / "dev_kmerGraph.txt").read_bytes() == (tmp_path / "host_kmerGraph.txt").read_bytes()
    assert (tmp_path / "dev_nodes.txt").read_bytes() == (tmp_path / "host_nodes.txt").read_bytes()


def test_long_reads_take_the_direct_build():
    """Reads longer than 16 kbp would leave the one-thread-per-read bucketed
    walker waiting on a few threads: the default builds them directly."""
    text = swapgb.synth_fasta(seed=71, genome_len=400_000, n_reads=60, read_len=20_000,
                              sub_rate=0.002)
    g = gpu_build(text, 31, 1)
    assert g.info()["algorithm"] == swapgb.ALGO_DIRECT
    assert_same_records(g, text, 31, 1)
    text = swapgb.synth_fasta(seed=72, genome_len=400_000, n_reads=600, read_len=2_000,
                              sub_rate=0.002)
    g = gpu_build(text, 31, 1)
    assert g.info()["algorithm"] == swapgb.ALGO_BUCKETED
    assert_same_records(g, text, 31, 1)


@pytest.mark.parametrize("shape", [1, 2, 3])
def test_scatter_shapes(shape, tmp_path):
    """The other block shapes of the two scatters (SWG_SCATTER_SHAPE, read
    once per process; 3 = level-2 chunks brought in by bulk copies into
    double-buffered shared memory) give the same graph."""
    import os
    import subprocess
    import sys
    fa = tmp_path / "reads.fa"
    swapgb.synth_fasta_file(str(fa), seed=81, genome_len=2_000_000, n_reads=400_000, read_len=100,
                            sub_rate=0.01, repeat_frac=0.05, tandem_frac=0.02)
    out = tmp_path / "graph.npz"
    code = ("import sys, numpy as np; sys.path.insert(0, %r); import swapgb\n"
            "t = open(%r, 'rb').read(); r = swapgb.reads_from_fasta(t, 31)\n"
            "g = swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=2, algorithm=swapgb.ALGO_BUCKETED), r)\n"
            "k, m = g.copy_out(sorted=True); np.savez(%r, k=k, m=m)\n"
            % (str(swapgb.PKG), str(fa), str(out)))
    env = dict(os.environ, SWG_SCATTER_SHAPE=str(shape))
    subprocess.run([sys.executable, "-c", code], env=env, check=True, timeout=300)
    got = np.load(out)
    okeys, omult = oracle.records(fa.read_bytes(), 31, 2)
    assert np.array_equal(got["k"], okeys) and np.array_equal(got["m"], omult)
