"""Full-scale property checks, beyond what the CPU restatement finishes in
seconds: the two independent counting schemes (one HBM table; shared-memory
buckets) must produce the same filtered graph, bit for bit, on a skewed input
large enough to take the bucketed path's 512-partition branch."""
import numpy as np
import pytest

import swapgb

pytestmark = pytest.mark.gpu


def test_large_skewed_input_bucketed_equals_direct():
    # a quarter of the 100 Mbp skewed workload: repeat families + tandem
    # repeats, 5M x 150 bp reads at 30x, k=31 c=3 (600M k-mer occurrences)
    text = swapgb.synth_fasta(seed=33, genome_len=25_000_000, repeat_frac=0.05, tandem_frac=0.02,
                              n_reads=5_000_000, read_len=150, sub_rate=0.005)
    reads = swapgb.reads_from_fasta(text, 31)
    del text
    gb = swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=3, algorithm=swapgb.ALGO_BUCKETED), reads)
    ib = gb.info()
    assert ib["occurrences"] > (400 << 20) and ib["partitions"] == 512, ib
    kb, mb = gb.copy_out(sorted=True)
    del gb
    gd = swapgb.Graph().build_reads(swapgb.Opts(k=31, cutoff=3, algorithm=swapgb.ALGO_DIRECT), reads)
    kd, md = gd.copy_out(sorted=True)
    assert gd.info()["distinct"] == ib["distinct"]
    assert kb.size == kd.size and np.array_equal(kb, kd)
    assert np.array_equal(mb, md)
    # saturation and the hot repeat keys are present
    assert (mb == 255).any()
