"""The serving loop: every job's distance matrix and join list are the same
alone and in a mix with other jobs, the same as the single-job context path,
and (for small jobs) the same as the oracle."""
import threading
import time

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import NWGError, Server, synth
from mestrado_gb300._native import NWG_ERR_INVALID, NWG_ERR_OOM

pytestmark = pytest.mark.gpu

JOIN_KEYS = ("i", "j", "node", "n", "len_i", "len_j", "q", "ti", "tj")


def _same_joins(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert tuple(x[k] for k in JOIN_KEYS) == tuple(y[k] for k in JOIN_KEYS)


def _mixed_jobs():
    jobs = [S for _, S in synth.serving_jobs(24, seed=11, n_hi=300)]
    # edges: one sequence, two, a family with long sequences (int32 lanes),
    # duplicates (exact NJ ties), ragged lengths
    jobs.append(synth.family(1, 50, seed=3))
    jobs.append(synth.family(2, 80, seed=4))
    jobs.append(synth.family(5, 3100, ps=0.05, pi=0.0, seed=5))
    dup = synth.family(12, 70, ps=0.02, pi=0.0, seed=6)
    jobs.append([dup[i] for i in range(len(dup))] + [dup[0], dup[0], dup[3]])
    jobs.append([b"W" * 700, b"ACDEFG", b"K" * 33, b"MKV" * 90])
    return jobs


def _run(srv, jobs, gap=0.0):
    ids = []
    for S in jobs:
        ids.append(srv.submit(S))
        if gap:
            time.sleep(gap)
    return [srv.wait(j, len(S)) for j, S in zip(ids, jobs)]


def test_serving_mix_equals_alone_and_context(ctx):
    jobs = _mixed_jobs()
    with Server(hbm_budget=4 << 30, max_batch_jobs=8) as srv:
        mixed = _run(srv, jobs)
    assert max(info["batch_jobs"] for _, _, info in mixed) > 1
    with Server(hbm_budget=4 << 30, max_batch_jobs=1) as srv:
        alone = _run(srv, jobs)
    for S, (Dm, Jm, im), (Da, Ja, ia) in zip(jobs, mixed, alone):
        assert im["status"] == 0 and ia["status"] == 0 and ia["batch_jobs"] == 1
        assert np.array_equal(Dm, Da)
        _same_joins(Jm, Ja)
        D = ctx.score_all(S)
        assert np.array_equal(Dm, D)
        if len(S) > 1:
            _same_joins(Jm, ctx.nj(D))
        assert im["nj_ambiguous_steps"] == 0 and im["nj_reference_identical"] == 1


def test_serving_batch_with_both_join_forms(ctx):
    # one batch holding jobs of up to 768 sequences (join loop in a cluster's
    # shared memory) and a job above that (join loop over L2): two launches in
    # one batch, every job as the context path gives it
    # (the first job usually goes alone; the big one, submitted last, joins
    # the small ones that arrive while the first batch runs)
    jobs = [S for _, S in synth.serving_jobs(6, seed=31, n_hi=400, median=60)]
    jobs.append(synth.family(900, 40, ps=0.1, pi=0.01, seed=7))
    with Server(hbm_budget=8 << 30, max_batch_jobs=8) as srv:
        res = _run(srv, jobs)
    assert max(info["batch_jobs"] for _, _, info in res) > 1
    for S, (D, J, info) in zip(jobs, res):
        assert info["status"] == 0
        Dc = ctx.score_all(S)
        assert np.array_equal(D, Dc)
        _same_joins(J, ctx.nj(Dc))


def test_serving_matches_oracle():
    jobs = [S for _, S in synth.serving_jobs(6, seed=21, n_hi=40, median=120)]
    with Server(max_batch_jobs=6) as srv:
        res = _run(srv, jobs)
    for S, (D, J, info) in zip(jobs, res):
        ref = O.score_all(S)
        assert np.array_equal(D, ref.astype(np.float32))
        oj, ost = O.nj(ref.astype(np.float32))
        _same_joins(J, oj)
        assert info["nj_tie_steps"] == ost["tie_steps"]
        assert info["nj_rebuilds"] == ost["rebuilds"]


def test_serving_wide_exact_ties():
    # jobs whose joins tie exactly on tens of thousands of pairs (420 copies
    # of one sequence; three sequences 140 times each)
    S = synth.family(4, 60, ps=0.02, pi=0.0, seed=41)
    jobs = [[S[0]] * 420, [S[k] for k in (1, 2, 3) for _ in range(140)]]
    with Server(hbm_budget=4 << 30, max_batch_jobs=4) as srv:
        res = _run(srv, jobs)
    for S, (D, J, info) in zip(jobs, res):
        assert info["status"] == 0
        assert np.array_equal(D, O.score_all(S).astype(np.float32))
        oj, ost = O.nj(D)
        _same_joins(J, oj)
        assert info["nj_ambiguous_steps"] == ost["ambiguous_steps"]
        assert info["nj_tie_steps"] == ost["tie_steps"]
        assert info["nj_reference_identical"] == (1 if ost["ambiguous_steps"] == 0 else 0)


def test_serving_admission_by_footprint(ctx):
    # a budget that holds about one 300-sequence job at a time: batches stay
    # small, results do not change
    jobs = [synth.family(n, 150, seed=30 + n) for n in (300, 280, 260, 40, 30)]
    budget = 300 * 300 * 4 + (1 << 19)
    with Server(hbm_budget=budget, max_batch_jobs=16) as srv:
        res = _run(srv, jobs)
    # 300 and 280 do not fit together; 260, 40 and 30 do
    assert [info["batch_jobs"] for _, _, info in res] == [1, 1, 3, 3, 3]
    for S, (D, J, info) in zip(jobs, res):
        assert np.array_equal(D, ctx.score_all(S))
        _same_joins(J, ctx.nj(D))


def test_serving_concurrent_submitters(ctx):
    jobs = [S for _, S in synth.serving_jobs(30, seed=41, n_hi=120)]
    out = [None] * len(jobs)
    with Server(max_batch_jobs=8) as srv:
        def worker(k0):
            for k in range(k0, len(jobs), 3):
                jid = srv.submit(jobs[k])
                out[k] = srv.wait(jid, len(jobs[k]))
        th = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    for S, (D, J, info) in zip(jobs, out):
        assert np.array_equal(D, ctx.score_all(S))
        assert info["latency_ms"] >= info["queue_ms"] >= 0


def test_serving_rejects():
    with Server(hbm_budget=1 << 20) as srv:
        with pytest.raises(NWGError) as e:
            srv.submit(synth.family(8200, 5, seed=1))
        assert e.value.status == NWG_ERR_INVALID
        with pytest.raises(NWGError) as e:
            srv.submit(synth.family(600, 20, seed=1))   # 1.4 MB matrix > 1 MB budget
        assert e.value.status == NWG_ERR_OOM
        with pytest.raises(NWGError) as e:
            srv.wait(12345, 3)
        assert e.value.status == NWG_ERR_INVALID


def test_waits_survive_rehashes_of_the_job_table(ctx):
    # One thread submits thousands of small jobs -- each insert may rehash the
    # server's job table -- while four threads wait on the jobs already
    # submitted.  Every wait returns its own job's result and releases it.
    import queue
    jobs = [synth.family(2 + k % 4, 24, seed=5000 + k) for k in range(4000)]
    q = queue.Queue()
    out = [None] * len(jobs)
    errors = []
    with Server(max_batch_jobs=64) as srv:
        def submitter():
            for k, S in enumerate(jobs):
                q.put((k, srv.submit(S)))
            for _ in range(4):
                q.put(None)

        def waiter():
            while True:
                item = q.get()
                if item is None:
                    return
                k, jid = item
                try:
                    out[k] = srv.wait(jid, len(jobs[k]))
                except Exception as e:  # noqa: BLE001 -- reported below
                    errors.append((k, repr(e)))

        th = [threading.Thread(target=submitter)] + [threading.Thread(target=waiter) for _ in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        with pytest.raises(NWGError):
            srv.wait(1, 2)          # released jobs are gone
    assert not errors, errors[:5]
    assert all(o is not None and o[2]["status"] == 0 for o in out)
    for k in range(0, len(jobs), 20):
        assert np.array_equal(out[k][0], ctx.score_all(jobs[k]))
