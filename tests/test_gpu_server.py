"""Request server: requests submitted while others run are batched together
(continuous batching); every result must equal the plain build of that
request alone; admission refuses requests larger than the budget."""
import random
import threading
import time

import numpy as np
import pytest

import swapgb

pytestmark = pytest.mark.gpu


def _requests():
    rng = random.Random(7)
    reqs = []
    for i in range(16):
        p = dict(seed=300 + i, genome_len=rng.choice([20_000, 50_000, 150_000]),
                 n_reads=rng.choice([2_000, 6_000, 12_000]), read_len=rng.choice([75, 100, 150]),
                 sub_rate=rng.uniform(0.001, 0.01))
        k, c = rng.choice([21, 25, 27, 31]), rng.choice([2, 3, 5])
        reqs.append((swapgb.synth_fasta(**p), k, c))
    return reqs


def _plain(text, k, c):
    g = swapgb.Graph()
    g.build_reads(swapgb.Opts(k=k, cutoff=c), swapgb.reads_from_fasta(text, k))
    return g.copy_out(sorted=True)


def test_mixed_requests_equal_plain_builds():
    reqs = _requests()
    reads = [swapgb.reads_from_fasta(t, k) for t, k, _ in reqs]
    srv = swapgb.Server(workers=2)
    tickets = [None] * len(reqs)

    def client(idx):
        for i in idx:
            time.sleep(random.Random(i).uniform(0, 0.004))
            tickets[i] = srv.submit(reads[i], reqs[i][1], reqs[i][2])

    th = [threading.Thread(target=client, args=(range(j, len(reqs), 2),)) for j in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, (text, k, c) in enumerate(reqs):
        srv.wait(tickets[i], 120.0)
        state, lat = srv.poll(tickets[i])
        assert state == swapgb.REQ_DONE and lat > 0
        keys, mult = srv.fetch(tickets[i])
        pk, pm = _plain(text, k, c)
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm), "request %d" % i
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["bytes_resident"] == 0 and st["bytes_reserved"] == 0
    srv.close()


def test_requests_arriving_during_a_build_join_the_next_batch():
    # one worker busy with a large request; the small requests submitted
    # meanwhile queue up and are built together as the next batch
    big = swapgb.reads_from_fasta(swapgb.synth_fasta(seed=9, genome_len=2_000_000, n_reads=1_500_000,
                                                     read_len=150, sub_rate=0.01), 31)
    reqs = _requests()[:8]
    small = [swapgb.reads_from_fasta(t, k) for t, k, _ in reqs]
    srv = swapgb.Server(workers=1)
    tb = srv.submit(big, 31, 5)
    ts = [srv.submit(r, k, c) for r, (_, k, c) in zip(small, reqs)]
    for t in [tb] + ts:
        srv.wait(t, 120.0)
    st = srv.stats()
    assert st["max_batch_requests"] >= 2 and st["batches"] < 1 + len(ts)
    for t, (text, k, c) in zip(ts, reqs):
        keys, mult = srv.fetch(t)
        pk, pm = _plain(text, k, c)
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm)
    srv.release(tb)
    srv.close()


def test_admission_refuses_oversized_requests():
    text, k, c = _requests()[0]
    r = swapgb.reads_from_fasta(text, k)
    srv = swapgb.Server(memory_budget=1 << 20)
    with pytest.raises(swapgb.SwgError) as e:
        srv.submit(r, k, c)
    assert e.value.status == 4  # SWG_ERR_ADMISSION
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_budget_for_one_request_at_a_time():
    reqs = _requests()[:4]
    reads = [swapgb.reads_from_fasta(t, k) for t, k, _ in reqs]
    occ = max(int((r.len.astype(np.int64) - k + 1).clip(min=0).sum()) for r, (_, k, _) in zip(reads, reqs))
    budget = int(occ / 0.6 * 32 * 1.5) + (64 << 20)
    srv = swapgb.Server(memory_budget=budget, workers=2)
    tickets = [srv.submit(r, k, c) for r, (_, k, c) in zip(reads, reqs)]
    for t, (text, k, c) in zip(tickets, reqs):
        srv.wait(t, 120.0)
        keys, mult = srv.fetch(t)
        pk, pm = _plain(text, k, c)
        assert np.array_equal(keys, pk) and np.array_equal(mult, pm)
    srv.close()
