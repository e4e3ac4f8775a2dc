"""The streamed FASTA build: a text of 96 MiB or more goes up in pieces, each
framed and scattered to the level-1 partitions as it lands, with the regions
sized from the first piece. Its graph must equal the one-shot build's (the
text copied whole, framed, then built; SWG_NO_STREAM selects it) bit for bit:
on plain inputs of 3 and 6 pieces (40 MiB each; the first framed with host
round trips, the rest on the device alone), with each algorithm, with a read
too long for the bucketed build in a later piece (the fallback), with the
multi-line quirk shifting the header/sequence alternation mid-text, with
later pieces denser than the first (framed again with round trips), on a
reused handle, and with the same errors for a NUL byte or an unpaired last
header."""
import os

import numpy as np
import pytest

import swapgb

pytestmark = pytest.mark.gpu

STREAM_MIN = 96 << 20


def synth(seed: int, n_reads: int, genome_len: int = 2_000_000) -> bytes:
    return swapgb.synth_fasta(seed=seed, genome_len=genome_len, n_reads=n_reads, read_len=100)


def build(text: bytes, opts: swapgb.Opts, streamed: bool, g: swapgb.Graph | None = None):
    if streamed:
        os.environ.pop("SWG_NO_STREAM", None)
    else:
        os.environ["SWG_NO_STREAM"] = "1"
    try:
        g = (g or swapgb.Graph()).build_fasta(opts, text)
    finally:
        os.environ.pop("SWG_NO_STREAM", None)
    keys, mult = g.copy_out(sorted=True)
    return g, keys, mult


def assert_same(text: bytes, opts: swapgb.Opts) -> dict:
    assert len(text) >= STREAM_MIN
    gs, ks, ms = build(text, opts, True)
    go, ko, mo = build(text, opts, False)
    si, oi = gs.info(), go.info()
    assert ks.size == ko.size and np.array_equal(ks, ko)
    assert np.array_equal(ms, mo)
    for key in ("occurrences", "distinct", "survivors"):
        assert si[key] == oi[key], (key, si, oi)
    return si


@pytest.fixture(scope="module")
def text2():
    # 1.1M x 100 bp reads: about 120 MB of text, three pieces
    return synth(41, 1_100_000)


def test_few_pieces_equal_one_shot(text2):
    info = assert_same(text2, swapgb.Opts(k=31, cutoff=5))
    assert info["algorithm"] == swapgb.ALGO_BUCKETED and info["survivors"] > 0
    assert info["estimate"] == 0  # the first piece's sample sized every region


def test_many_pieces_equal_one_shot_and_host_framing():
    text = synth(42, 2_600_000, genome_len=5_000_000)  # about 287 MB: six pieces
    assert len(text) >= 6 * (40 << 20)
    opts = swapgb.Opts(k=21, cutoff=2)
    assert assert_same(text, opts)["estimate"] == 0
    _, ks, ms = build(text, opts, True)
    gh = swapgb.Graph().build_reads(opts, swapgb.reads_from_fasta(text, 21))
    kh, mh = gh.copy_out(sorted=True)
    assert np.array_equal(ks, kh) and np.array_equal(ms, mh)


@pytest.mark.parametrize("algo", [swapgb.ALGO_BUCKETED, swapgb.ALGO_DIRECT, swapgb.ALGO_PARTITIONED])
def test_each_algorithm(text2, algo):
    assert_same(text2, swapgb.Opts(k=31, cutoff=3, algorithm=algo))


def test_minimizer_order_falls_back(text2):
    assert_same(text2, swapgb.Opts(k=31, cutoff=3, read_order=swapgb.ORDER_MINIMIZER))


def test_long_read_in_a_later_piece_falls_back(text2):
    rng = np.random.default_rng(3)
    long_read = bytes(np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 20_000)])
    text = text2 + b">long\n" + long_read + b"\n"
    info = assert_same(text, swapgb.Opts(k=31, cutoff=1))
    assert info["algorithm"] != swapgb.ALGO_BUCKETED  # the one-shot default takes the direct build


def test_multiline_record_shifts_the_alternation(text2):
    # a sequence split over two lines: from there on the reference reads
    # every header as a sequence and every sequence as a header (one more
    # line at the end keeps the line count even: the old last sequence line
    # is that record's header)
    half = len(text2) // 2
    cut = text2.index(b"\n>", half) + 1
    ml = b">ml\n" + b"ACGTTGCA" * 10 + b"\n" + b"TTGCAACG" * 10 + b"\n"
    text = text2[:cut] + ml + text2[cut:] + b"GATTACA" * 12 + b"\n"
    opts = swapgb.Opts(k=19, cutoff=1)
    shifted = assert_same(text, opts)
    plain = build(text2, opts, True)[0].info()
    # the second half's sequences are headers now, its headers too short to count
    assert shifted["occurrences"] < 0.6 * plain["occurrences"]


def test_handle_reuse_across_streamed_builds(text2):
    opts = swapgb.Opts(k=31, cutoff=2)
    other = synth(43, 1_000_000, genome_len=3_000_000)
    g, _, _ = build(other, opts, True)
    g, ks, ms = build(text2, opts, True, g)
    _, ko, mo = build(text2, opts, False)
    assert np.array_equal(ks, ko) and np.array_equal(ms, mo)


def test_errors_match_one_shot(text2):
    bad_nul = text2[:-50] + b"\x00" + text2[-49:]
    unpaired = text2 + b">no_sequence\n"
    for bad in (bad_nul, unpaired):
        for streamed in (True, False):
            with pytest.raises(swapgb.SwgError) as e:
                build(bad, swapgb.Opts(k=31, cutoff=5), streamed)
            assert e.value.status == 1


def test_sample_miss_recounts_exactly(text2):
    # 200k reads of one dinucleotide repeat, all in the second piece: the
    # first piece's sample cannot see the two hot k-mers, their bucket
    # outgrows its region, and the streamed build recounts with exact counts
    hot = b"".join(b">t%d\n" % i + b"AC" * 50 + b"\n" for i in range(200_000))
    text = text2 + hot
    opts = swapgb.Opts(k=31, cutoff=3)
    info = assert_same(text, opts)
    assert info["estimate"] == 1  # the exact-count rerun ran
    gs, ks, ms = build(text, opts, True)
    assert (ms == 255).any()  # the hot k-mers saturate


def test_denser_later_pieces_frame_again():
    """Pieces after the first are framed on the device into capacities
    estimated from the first piece. Here the first piece holds 250 bp reads
    and the rest 40 bp reads (about five times the newlines per byte): the
    estimate is outgrown, the build frames the text again with host round
    trips, and the graph still equals the one-shot build's."""
    long_part = swapgb.synth_fasta(seed=51, genome_len=3_000_000, n_reads=140_000, read_len=250)
    short_part = swapgb.synth_fasta(seed=52, genome_len=3_000_000, n_reads=2_000_000, read_len=40)
    text = long_part + short_part
    assert len(text) >= STREAM_MIN and len(long_part) > len(text) // 4  # the first piece: long reads only
    assert_same(text, swapgb.Opts(k=21, cutoff=2))


def _to_host(g: swapgb.Graph, opts: swapgb.Opts, text: bytes, keys, mult, cap: int) -> tuple[int, int]:
    import ctypes as C
    h = np.frombuffer(text, dtype=np.uint8)
    n = C.c_uint64()
    st = swapgb.lib().swg_graph_build_fasta_to_host(g._h, C.byref(opts), h.ctypes.data, h.size, keys, mult,
                                                     cap, C.byref(n))
    return st, n.value


@pytest.mark.parametrize("case", ["streamed", "one_shot", "hot_keys", "direct"])
def test_build_to_host_equals_build_then_copy(case, text2):
    """swg_graph_build_fasta_to_host into pinned arrays (the bucket count
    writes each bucket's survivors there as it goes) equals
    swg_graph_build_fasta + swg_graph_copy_out, as a set; twice in a row on
    one handle; through the streamed and the one-shot framing, with buckets
    too large for shared memory (the global-table path), and with the direct
    algorithm (copied after the build)."""
    import torch
    opts = swapgb.Opts(k=31, cutoff=5)
    text = text2
    if case == "one_shot":
        text = synth(43, 200_000)
    elif case == "hot_keys":
        reads = ["A" * 250, "AC" * 125] * 30000 + ["ACGTTGCA" * 20] * 500
        text = "".join(">h%d\n%s\n" % (i, r) for i, r in enumerate(reads)).encode() + synth(44, 100_000)
        opts = swapgb.Opts(k=21, cutoff=2)
    elif case == "direct":
        opts = swapgb.Opts(k=31, cutoff=5, algorithm=swapgb.ALGO_DIRECT)
    want_g = swapgb.Graph().build_fasta(opts, text)
    wk, wm = want_g.copy_out(sorted=True)
    cap = wk.size + 16
    keys = torch.zeros(cap, dtype=torch.int64).pin_memory()
    mult = torch.zeros(cap * 8, dtype=torch.uint8).pin_memory()
    g = swapgb.Graph()
    for _ in range(2):
        st, n = _to_host(g, opts, text, keys.data_ptr(), mult.data_ptr(), cap)
        assert st == 0, swapgb.lib().swg_last_error().decode()
        assert n == wk.size
        k = keys.numpy().view(np.uint64)[:n]
        m = mult.numpy().reshape(-1, 8)[:n]
        o = np.argsort(k, kind="stable")
        assert np.array_equal(k[o], wk) and np.array_equal(m[o], wm)
        dk, dm = g.copy_out(sorted=True)  # the graph stays on the device too
        assert np.array_equal(dk, wk) and np.array_equal(dm, wm)
    # too small: the count needed comes back
    st, n = _to_host(g, opts, text, keys.data_ptr(), mult.data_ptr(), max(1, wk.size // 2))
    assert st == 1 and n == wk.size


def test_build_to_host_pageable_arrays(text2):
    """Arrays the device cannot address (pageable numpy memory): the graph is
    copied after the build, with the same result."""
    opts = swapgb.Opts(k=31, cutoff=5)
    wk, wm = swapgb.Graph().build_fasta(opts, text2).copy_out(sorted=True)
    keys = np.zeros(wk.size, dtype=np.uint64)
    mult = np.zeros((wk.size, 8), dtype=np.uint8)
    st, n = _to_host(swapgb.Graph(), opts, text2, keys.ctypes.data, mult.ctypes.data, wk.size)
    assert st == 0 and n == wk.size
    o = np.argsort(keys, kind="stable")
    assert np.array_equal(keys[o], wk) and np.array_equal(mult[o], wm)
