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


def test_full_skewed_workload_builds_and_merges_agree():
    """The full 100 Mbp skewed workload (20M x 150 bp reads at 30x, repeat
    families + tandem repeats, k=31 c=3; 2.4G k-mer occurrences, ~96M
    k-molecules kept), too large for the CPU restatement here: the bucketed
    and the direct build must agree bit for bit, and so must the merged
    graphs computed from their (differently ordered) outputs."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    work, k, c, _ = bench.CONFIGS[3]
    reads = swapgb.reads_from_fasta(swapgb.synth_fasta(**work), k)
    gb = swapgb.Graph().build_reads(swapgb.Opts(k=k, cutoff=c, algorithm=swapgb.ALGO_BUCKETED), reads)
    ib = gb.info()
    assert ib["algorithm"] == swapgb.ALGO_BUCKETED and ib["occurrences"] > 2_000_000_000, ib
    gb.merge()
    tb, mi = gb.merged_text(), gb.merge_info()
    kb, mb = gb.copy_out(sorted=True)
    del gb
    gd = swapgb.Graph().build_reads(swapgb.Opts(k=k, cutoff=c, algorithm=swapgb.ALGO_DIRECT), reads)
    del reads
    assert gd.info()["distinct"] == ib["distinct"]
    kd, md = gd.copy_out(sorted=True)
    assert kb.size == kd.size and np.array_equal(kb, kd) and np.array_equal(mb, md)
    del kd, md
    gd.merge()
    assert gd.merged_text() == tb
    # every node left has other than one arc per side, or is a self-looped
    # node or a cut cycle's survivor
    one_each = int(np.count_nonzero(((mb[:, :4] != 0).sum(1) == 1) & ((mb[:, 4:] != 0).sum(1) == 1)))
    assert mi["nodes"] >= kb.size - one_each
    assert mi["nodes"] == tb.count(b"\n") - 1


@pytest.mark.parametrize("config", [2, 3])
def test_full_workloads_match_the_restatement(config):
    """Workload 2 (5 Mbp, 2.5M x 100 bp, k31 c5) and workload 3 (the 100 Mbp
    skewed genome, 20M x 150 bp, k31 c3) at full size: the default build
    equals the CPU restatement (all host cores) bit for bit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    import oracle
    work, k, c, _ = bench.CONFIGS[config]
    text = swapgb.synth_fasta(**work)
    g = swapgb.Graph().build_fasta(swapgb.Opts(k=k, cutoff=c), text)
    keys, mult = g.copy_out(sorted=True)
    del g
    okeys, omult = oracle.records(text, k, c)
    del text
    assert keys.size == okeys.size and np.array_equal(keys, okeys)
    assert np.array_equal(mult, omult)
