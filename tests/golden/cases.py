"""Parity cases: hand-written known-answer inputs and seeded synthetic inputs.

The reference has no tests and no data; these inputs were written for this
project. The reference's outputs on them are stored by make_golden.py.
"""
from __future__ import annotations

import random

from swapgb import synth_fasta


def _rand_seq(rng: random.Random, n: int) -> str:
    return "".join(rng.choice("ACGT") for _ in range(n))


def _revcomp(s: str) -> str:
    return s[::-1].translate(str.maketrans("ACGT", "TGCA"))


def _reads_from(genome: str, rng: random.Random, n: int, L: int, err: float) -> list[str]:
    out = []
    for _ in range(n):
        st = rng.randint(0, len(genome) - L)
        r = genome[st:st + L]
        if rng.random() < 0.5:
            r = _revcomp(r)
        r = list(r)
        for j in range(L):
            if rng.random() < err:
                r[j] = rng.choice("ACGT".replace(r[j], ""))
        out.append("".join(r))
    return out


def _fasta(reads: list[str], nl: str = "\n") -> bytes:
    return "".join(">r%d%s%s%s" % (i, nl, s, nl) for i, s in enumerate(reads)).encode()


def _kat_cases() -> list[dict]:
    rng = random.Random(20261203)
    g = _rand_seq(rng, 1500)
    base = _reads_from(g, rng, 120, 60, 0.01)
    cases = []
    cases.append(dict(name="orient_k19", k=19, c=1, text=_fasta(base),
                      why="both strands: all four orientation cases of kmerGraph.cpp:261-296"))
    cases.append(dict(name="orient_k19_c0", k=19, c=0, text=_fasta(base),
                      why="c=0: only all-zero keys are dropped (graph.cpp:1106-1108)"))
    cases.append(dict(name="orient_k31_c3", k=31, c=3, text=_fasta(base),
                      why="largest k, cutoff removes low-count slots"))
    odd = [s for s in base[:30]]
    odd[0] = odd[0][:10] + "NNNN" + odd[0][14:]
    odd[1] = odd[1].lower()
    odd[2] = odd[2][:5] + "RYKM-.*" + odd[2][12:]
    odd[3] = odd[3][:18]            # shorter than k: skipped
    odd[4] = odd[4][:19]            # exactly k: one key with an all-zero mask
    odd[5] = odd[5][:20]            # k+1: one adjacency
    cases.append(dict(name="normalise_k19", k=19, c=0, text=_fasta(odd),
                      why="N/lowercase/IUPAC -> A (kmerGraph.cpp:228-233), short reads, L==k, L==k+1"))
    poly = ["A" * 60, "T" * 45, "AC" * 30, "ACG" * 25, "AT" * 30, "CG" * 25, "ACGT" * 20]
    cases.append(dict(name="tandem_k21", k=21, c=1, text=_fasta(poly * 3),
                      why="self-adjacent and palindromic-unit k-mers, equal keys inside one read"))
    sat = [base[7]] * 300 + base[:20]
    cases.append(dict(name="saturate_k21", k=21, c=2, text=_fasta(sat),
                      why="uint8 multiplicities saturate at 255 (graph.cpp:1076)"))
    cases.append(dict(name="saturate_k21_c255", k=21, c=255, text=_fasta(sat),
                      why="cutoff at the saturation value keeps only saturated slots"))
    cases.append(dict(name="cutoff256_k21", k=21, c=256, text=_fasta(sat),
                      why="cutoff above 255 removes every k-molecule"))
    cases.append(dict(name="crlf_k19", k=19, c=1, text=_fasta(base[:40], nl="\r\n"),
                      why="CRLF files: the trailing '\\r' is part of the sequence line and becomes 'A'"))
    multi = []
    for i, s in enumerate(base[:26]):  # even line count: the last record is complete
        multi.append(">m%d\n%s\n%s\n" % (i, s[:30], s[30:]))
    cases.append(dict(name="multiline_k19", k=19, c=0, text="".join(multi).encode(),
                      why="multi-line records: lines are taken as header/sequence alternately"))
    # two blank lines keep the total line count even (an odd count leaves a
    # header without its sequence line, which the reference never finishes)
    blank = _fasta(base[:20]).decode().replace(">r5\n", "\n>r5\n").replace(">r12\n", "\n>r12\n")
    blank = blank.encode()
    cases.append(dict(name="blankline_k19", k=19, c=0, text=blank,
                      why="a blank line shifts the header/sequence alternation"))
    # Bytes before the first '>' are not a parity case: the reference adds
    # their count to the bytes left to read (kmerGraph.cpp:121-125), reads
    # that far past the end of the file and never finishes.
    hdr = "".join(">%s\n%s\n" % (h, s) for h, s in zip(["", ">>", "x y z", "r>q"] * 5, base[:20]))
    cases.append(dict(name="headers_k19", k=19, c=1, text=hdr.encode(),
                      why="empty and '>'-laden header lines"))
    lens = [19, 20, 23, 47, 64, 65, 100, 129, 250, 333]
    ragged = [_rand_seq(rng, L) for L in lens]
    ragged += [g[i:i + L] for i, L in zip(range(0, 1400, 137), lens)]
    cases.append(dict(name="ragged_k25", k=25, c=1, text=_fasta(ragged),
                      why="ragged read lengths, word-boundary offsets of the packed stream"))
    return cases


KAT_CASES = _kat_cases()

# Seeded synthetic cases; `parts` concatenates several generator runs (ragged
# read lengths). The first is the CPU-runnable workload itself: a 1 Mbp
# uniform genome, 300k 100 bp reads from both strands, 0.5% substitutions,
# k=21, c=2.
SYNTH_CASES = [
    dict(name="c1_full", k=21, c=2, why="1 Mbp genome, 30x 100 bp reads, 0.5% subs, k21 c2",
         params=[dict(seed=1, genome_len=1000000, n_reads=300000, read_len=100, sub_rate=0.005)]),
    dict(name="c1_small", k=21, c=2, why="reduced c1",
         params=[dict(seed=2, genome_len=20000, n_reads=6000, read_len=100, sub_rate=0.005)]),
    dict(name="c2_small", k=31, c=5, why="reduced c2: 1% subs + 0.1% indels, 50x, k31 c5",
         params=[dict(seed=3, genome_len=50000, n_reads=25000, read_len=100, sub_rate=0.01,
                      indel_rate=0.001)]),
    dict(name="c3_small", k=31, c=3,
         why="reduced c3: repeat families + tandem repeats, 150 bp at 30x, k31 c3",
         params=[dict(seed=4, genome_len=200000, repeat_frac=0.05, tandem_frac=0.02,
                      n_reads=40000, read_len=150, sub_rate=0.005)]),
    dict(name="c4_ragged", k=27, c=3, why="read lengths 75/100/150/250 in one file, k27 c3",
         params=[dict(seed=5, genome_len=30000, n_reads=6000, read_len=75, sub_rate=0.003),
                 dict(seed=6, genome_len=30000, n_reads=4000, read_len=100, sub_rate=0.008),
                 dict(seed=7, genome_len=30000, n_reads=3000, read_len=150, sub_rate=0.001),
                 dict(seed=8, genome_len=30000, n_reads=2000, read_len=250, sub_rate=0.01)]),
    dict(name="k25_c1", k=25, c=1, why="k25, cutoff 1",
         params=[dict(seed=9, genome_len=40000, n_reads=8000, read_len=120, sub_rate=0.01)]),
]


def synth_text(case: dict) -> bytes:
    return b"".join(synth_fasta(**p) for p in case["params"])


def _circular_reads(rng: random.Random, genome_len: int, n: int, L: int) -> list[str]:
    g = _rand_seq(rng, genome_len)
    gg = g + g[:L]  # reads wrap around the end: a circular genome
    out = []
    for _ in range(n):
        st = rng.randrange(genome_len)
        r = gg[st:st + L]
        out.append(_revcomp(r) if rng.random() < 0.5 else r)
    return out


def _merge_cases() -> list[dict]:
    rng = random.Random(1392)
    cycles = (_circular_reads(rng, 500, 200, 80) + ["ACGTT" * 30] * 5 + ["AC" * 50] * 4 +
              _circular_reads(rng, 1200, 400, 100))
    return [
        dict(name="merge_errors_k21", k=21, c=1, why="1% errors kept by c=1: many tips and bubbles",
             params=[dict(seed=31, genome_len=6000, n_reads=1500, read_len=100, sub_rate=0.01)]),
        dict(name="merge_repeats_k31", k=31, c=2, why="repeat families and tandem repeats, k31",
             params=[dict(seed=32, genome_len=8000, repeat_frac=0.1, tandem_frac=0.05, n_reads=2000,
                          read_len=150, sub_rate=0.005)]),
        dict(name="merge_cycles_k23", k=23, c=3, text=_fasta(cycles),
             why="isolated cycles: two circular genomes and two tandem repeats"),
        dict(name="merge_k19_c0", k=19, c=0, why="k19, c=0, indels",
             params=[dict(seed=33, genome_len=3000, n_reads=800, read_len=75, sub_rate=0.02,
                          indel_rate=0.002)]),
    ]


# Merge stage (graph.cpp:1392-1566) cases; make_merge_golden.py stores the
# reference's visiting order and a hash of its -d output for each.
MERGE_CASES = _merge_cases()


def case_text(case: dict) -> bytes:
    return case["text"] if "text" in case else synth_text(case)
