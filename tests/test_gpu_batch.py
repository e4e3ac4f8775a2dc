"""Batched build: many samples with uneven sizes, read lengths, k and cutoff
in one build; every sample's result must equal the plain build of that
sample alone (and the CPU restatement), bit for bit."""
import numpy as np
import pytest

import oracle
import swapgb

pytestmark = pytest.mark.gpu

SAMPLES = [  # (generator parameters, k, cutoff)
    (dict(seed=101, genome_len=50_000, n_reads=8_000, read_len=75, sub_rate=0.002), 27, 3),
    (dict(seed=102, genome_len=200_000, n_reads=30_000, read_len=150, sub_rate=0.01), 27, 3),
    (dict(seed=103, genome_len=80_000, n_reads=4_000, read_len=250, sub_rate=0.005), 31, 5),
    (dict(seed=104, genome_len=30_000, n_reads=9_000, read_len=100, sub_rate=0.001,
          indel_rate=0.001), 21, 2),
    (dict(seed=105, genome_len=120_000, repeat_frac=0.05, tandem_frac=0.02, n_reads=20_000,
          read_len=150, sub_rate=0.005), 27, 3),
    (dict(seed=106, genome_len=10_000, n_reads=2_000, read_len=100, sub_rate=0.0), 19, 0),
    (dict(seed=107, genome_len=60_000, n_reads=15_000, read_len=100, sub_rate=0.01), 25, 1),
]


def _plain(text, k, c):
    g = swapgb.Graph()
    g.build_reads(swapgb.Opts(k=k, cutoff=c), swapgb.reads_from_fasta(text, k))
    return g.copy_out(sorted=True)


@pytest.fixture(scope="module")
def texts():
    return [swapgb.synth_fasta(**p) for p, _, _ in SAMPLES]


def test_batch_equals_plain_builds(texts):
    reads = [swapgb.reads_from_fasta(t, k) for t, (_, k, _) in zip(texts, SAMPLES)]
    # a sample whose reads are all shorter than k, and an empty one
    short = swapgb.reads_from_fasta(b">a\nACGTACGT\n>b\nACG\n", 21)
    batch = [(r, k, c) for r, (_, k, c) in zip(reads, SAMPLES)] + [(short, 21, 2)]
    g = swapgb.Graph()
    g.build_batch(swapgb.Opts(), batch)
    assert g.batch_size() == len(batch)
    for i, (text, (_, k, c)) in enumerate(zip(texts, SAMPLES)):
        keys, mult = g.batch_copy_out(i)
        pk, pm = _plain(text, k, c)
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm), "sample %d" % i
        if i in (0, 3, 5):
            ok, om = oracle.records(text, k, c)
            assert np.array_equal(keys, ok) and np.array_equal(mult, om)
        occ, distinct, surv = g.batch_info(i)
        assert surv == keys.size and distinct >= surv and occ > 0
    assert g.batch_info(len(batch) - 1) == (0, 0, 0)


def test_batch_handle_reuse_and_single_sample_calls(texts):
    g = swapgb.Graph()
    r0 = swapgb.reads_from_fasta(texts[1], 27)
    g.build_batch(swapgb.Opts(), [(r0, 27, 3)])
    with pytest.raises(swapgb.SwgError):
        g.size()  # single-sample accessors refuse a batched result
    r1 = swapgb.reads_from_fasta(texts[2], 31)
    r2 = swapgb.reads_from_fasta(texts[4], 27)
    g.build_batch(swapgb.Opts(load_factor=0.8), [(r2, 27, 3), (r1, 31, 5)])
    for i, (t, k, c) in enumerate(((texts[4], 27, 3), (texts[2], 31, 5))):
        keys, mult = g.batch_copy_out(i)
        pk, pm = _plain(t, k, c)
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm)
    # the same handle then runs a plain build again
    g.build_reads(swapgb.Opts(k=27, cutoff=3), r0)
    keys, mult = g.copy_out()
    pk, pm = _plain(texts[1], 27, 3)
    assert np.array_equal(keys, pk) and np.array_equal(mult, pm)


# samples whose k leaves room for the sample tag above the k-mer (k <= 27):
# the default batch runs them through one tagged bucketed build
TAGGED = [i for i, (_, k, _) in enumerate(SAMPLES) if k <= 27]


@pytest.mark.parametrize("algo", [swapgb.ALGO_DEFAULT, swapgb.ALGO_DIRECT])
def test_tagged_batch_equals_plain_builds(texts, algo):
    short = swapgb.reads_from_fasta(b">a\nACGTACGT\n>b\nACG\n", 21)
    batch = [(swapgb.reads_from_fasta(texts[i], SAMPLES[i][1]), SAMPLES[i][1], SAMPLES[i][2])
             for i in TAGGED] + [(short, 21, 2)]
    g = swapgb.Graph()
    g.build_batch(swapgb.Opts(algorithm=algo), batch)
    assert g.info()["algorithm"] == (swapgb.ALGO_BUCKETED if algo == swapgb.ALGO_DEFAULT
                                     else swapgb.ALGO_DIRECT)
    for j, i in enumerate(TAGGED):
        keys, mult = g.batch_copy_out(j)
        pk, pm = _plain(texts[i], SAMPLES[i][1], SAMPLES[i][2])
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm), "sample %d" % i
        occ, distinct, surv = g.batch_info(j)
        assert surv == keys.size and distinct >= surv and occ > 0
    assert g.batch_info(len(batch) - 1) == (0, 0, 0)


def test_tagged_batch_many_samples_and_overflow():
    """300 samples (9 tag bits, k=21), one of them a single hot k-mer whose
    bucket no shared-memory table holds (the global-table path): every sample
    still equals its own plain build."""
    hot = "".join(">h%d\n%s\n" % (i, "A" * 150) for i in range(3000)).encode()
    texts = [swapgb.synth_fasta(seed=500 + i, genome_len=3_000 + 97 * i, n_reads=300 + 5 * i,
                                read_len=(75, 100, 150)[i % 3], sub_rate=0.005) for i in range(299)]
    texts.insert(137, hot)
    batch = [(swapgb.reads_from_fasta(t, 21), 21, 2 + (i % 3)) for i, t in enumerate(texts)]
    g = swapgb.Graph()
    g.build_batch(swapgb.Opts(), batch)
    info = g.info()
    assert info["algorithm"] == swapgb.ALGO_BUCKETED and info["waves"] >= 1, info
    for i in list(range(0, 300, 23)) + [137, 299]:
        keys, mult = g.batch_copy_out(i)
        pk, pm = _plain(texts[i], 21, 2 + (i % 3))
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm), "sample %d" % i
    ok, om = oracle.records(texts[137], 21, 2 + (137 % 3))
    keys, mult = g.batch_copy_out(137)
    assert np.array_equal(keys, ok) and np.array_equal(mult, om)


def test_batched_workload_samples_equal_the_restatement():
    """32 samples of the batched workload's distribution (8 per read length:
    75, 100, 150 and 250 bp; genomes 50 kbp-2 Mbp at 10-60x), built as one
    batch with k=27, c=3; each sample's k-molecules and multiplicities equal
    the CPU restatement of the reference on that sample alone
    (kmerGraph.cpp:95-310, graph.cpp:1049-1114), bit for bit."""
    specs = swapgb.batch_workload_specs(256, seed=4)
    chosen = []
    for L in (75, 100, 150, 250):
        chosen += [p for p in specs if p["read_len"] == L][:8]
    assert len(chosen) == 32
    texts = [swapgb.synth_fasta(**p) for p in chosen]
    g = swapgb.Graph()
    g.build_batch(swapgb.Opts(), [(swapgb.reads_from_fasta(t, 27), 27, 3) for t in texts])
    assert g.batch_size() == 32
    for i, t in enumerate(texts):
        keys, mult = g.batch_copy_out(i)
        ok, om = oracle.records(t, 27, 3)
        assert np.array_equal(keys, ok) and np.array_equal(mult, om), "sample %d (%s)" % (i, chosen[i])
