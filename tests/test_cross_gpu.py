"""Cross RMSD (query sets against a resident database) and the serving loop.

Parity: every entry against the FP64 Kabsch oracle (ABS_TOL nm), rows
against the reference's md.rmsd(db[a:b], queries, k) semantics through the
CPU oracle; serving: each request's result is bit-identical alone and in a
mix (tolerance 0), and matches the oracle."""
import numpy as np
import pytest

from conftest import ABS_TOL, assert_parity
from mdtraj_gb300 import cross, serving, synth
from oracle import cpu, fp64

pytestmark = pytest.mark.gpu


def chain_db(F, A, seed):
    return synth.gaussian_chain(F, A, seed=seed).numpy()


def oracle_block(db, queries, a, b):
    return np.stack([fp64.kabsch_rmsd(db[a:b], q) for q in queries])


@pytest.mark.parametrize("method", ["tensor", "fp32"])
@pytest.mark.parametrize("F,A,Q,rng_", [(500, 300, 19, (0, 500)), (257, 61, 5, (3, 250)), (90, 130, 81, (40, 41)),
                                        (64, 7, 1, (0, 64))])
def test_cross_matches_fp64(cuda, method, F, A, Q, rng_):
    db = chain_db(F, A, seed=F + A)
    idx = np.random.default_rng(Q).integers(0, F, Q)
    q = synth.perturbed_queries(db, idx, seed=Q)
    q[0] = db[idx[0]]                    # an exact database frame: rmsd 0 at idx[0]
    a, b = rng_
    got = cross.cross_rmsd(db, q, db_range=(a, b), method=method)
    assert got.shape == (Q, b - a) and got.dtype == np.float32
    want = oracle_block(db, q, a, b)
    assert_parity(got.ravel(), want.ravel(), what=f"cross {method} F={F} A={A} Q={Q}")
    if a <= idx[0] < b:
        assert got[0, idx[0] - a] <= 1e-5


def test_cross_rows_match_reference_md_rmsd(cuda):
    db = chain_db(400, 120, seed=5)
    q = synth.perturbed_queries(db, [3, 99, 250], seed=1)
    got = cross.cross_rmsd(db, q, db_range=(50, 350), method="tensor")
    ref = cpu.best_available()
    for k in range(3):
        target = np.ascontiguousarray(db[50:350])
        row = ref.md_rmsd(target, np.ascontiguousarray(q[k]))
        want = fp64.kabsch_rmsd(db[50:350], q[k])
        assert_parity(got[k], want, row, what=f"row {k} vs reference md.rmsd")


def test_cross_tensor_equals_fp32(cuda):
    db = chain_db(700, 300, seed=11)
    q = synth.perturbed_queries(db, np.arange(0, 700, 37), seed=2)
    t = cross.cross_rmsd(db, q, method="tensor")
    f = cross.cross_rmsd(db, q, method="fp32")
    assert np.abs(t - f).max() <= 2 * ABS_TOL


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_cross_many_requests_share_tiles(cuda, method):
    import torch

    from mdtraj_gb300 import _device as D

    F, A = 600, 96
    db = chain_db(F, A, seed=7)
    dbs = cross.FrameSet.from_frames(db)
    rng = np.random.default_rng(4)
    sizes = [1, 3, 80, 17, 2, 160]
    ranges = [(0, F), (10, 11), (100, 580), (0, 300), (599, 600), (250, 400)]
    qs = [synth.perturbed_queries(db, rng.integers(0, F, n), seed=n) for n in sizes]
    cap = sum(sizes) + 13
    qset = cross.FrameSet(cap, A)
    pool0, p = [], 5
    for q in qs:
        qset.prepare(torch.from_numpy(q.reshape(len(q), -1)).to(cuda), p)
        pool0.append(p)
        p += len(q)
    outs = [torch.full((len(q), b - a), -1.0, device=cuda) for q, (a, b) in zip(qs, ranges)]
    table = cross.request_table([(o.data_ptr(), p0, len(q), a, b) for o, p0, q, (a, b) in
                                 zip(outs, pool0, qs, ranges)])
    ws = cross.CrossWorkspace(cuda).get(F, cap, len(qs))
    cross.cross_launch(dbs, F, qset, table, len(qs), method, ws, D.stream_handle())
    cross.cross_status(ws)
    for o, q, (a, b) in zip(outs, qs, ranges):
        assert_parity(o.cpu().numpy().ravel(), oracle_block(db, q, a, b).ravel(), what=f"request {a}:{b}")


def test_cross_rejects_overlapping_query_rows(cuda):
    import torch

    from mdtraj_gb300 import _device as D

    db = chain_db(50, 20, seed=1)
    dbs = cross.FrameSet.from_frames(db)
    qset = cross.FrameSet(10, 20)
    out = torch.empty(100, device=cuda)
    table = cross.request_table([(out.data_ptr(), 0, 4, 0, 10), (out.data_ptr(), 3, 2, 0, 10)])
    ws = cross.CrossWorkspace(cuda).get(50, 10, 2)
    with pytest.raises(ValueError, match="share query row"):
        cross.cross_launch(dbs, 50, qset, table, 2, "tensor", ws, D.stream_handle())


def make_requests(db, n, seed, max_q=64, rate=2000.0):
    rng = np.random.default_rng(seed)
    F = db.shape[0]
    reqs, t = [], 0.0
    for k in range(n):
        Q = int(np.clip(np.rint(synth.log_uniform(rng, 1, max_q, 1)[0]), 1, max_q))
        if rng.random() < 0.5:
            a, b = 0, F
        else:
            ln = int(rng.integers(max(1, F // 20), F + 1))
            a = int(rng.integers(0, F - ln + 1))
            b = a + ln
        q = synth.perturbed_queries(db, rng.integers(0, F, Q), seed=seed * 1000 + k)
        t += rng.exponential(1.0 / rate)
        reqs.append(serving.Request(queries=q, db0=a, db1=b, arrival=t, rid=k))
    return reqs


def clone(reqs):
    return [serving.Request(queries=r.queries, db0=r.db0, db1=r.db1, arrival=r.arrival, rid=r.rid) for r in reqs]


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_serving_alone_equals_mix(cuda, method):
    db = chain_db(3000, 300, seed=21)
    dbs = cross.FrameSet.from_frames(db)
    reqs = make_requests(db, 24, seed=3)
    server = serving.RmsdServer(dbs, method=method, query_capacity=1024, slots=3)
    # all at once: large mixed batches
    mixed = {r.rid: r.result for r in server.serve(clone(reqs), realtime=False)}
    assert max(server.batch_sizes) > 1
    # real-time Poisson arrivals: batches form as requests arrive
    timed = {r.rid: r.result for r in server.serve(clone(reqs), realtime=True)}
    # one request per launch
    alone_server = serving.RmsdServer(dbs, method=method, query_capacity=1024, slots=1, max_batch_requests=1)
    alone = {r.rid: r.result for r in alone_server.serve(clone(reqs), realtime=False)}
    assert max(alone_server.batch_sizes) == 1
    for r in reqs:
        np.testing.assert_array_equal(mixed[r.rid], alone[r.rid], err_msg=f"request {r.rid} mixed vs alone")
        np.testing.assert_array_equal(timed[r.rid], alone[r.rid], err_msg=f"request {r.rid} timed vs alone")
    for r in reqs[:6]:
        assert_parity(alone[r.rid].ravel(), oracle_block(db, r.queries, r.db0, r.db1).ravel(),
                      what=f"request {r.rid}")


def test_serving_budget_gates_admission(cuda):
    db = chain_db(2000, 64, seed=2)
    reqs = make_requests(db, 12, seed=5, max_q=16)
    biggest = max(r.result_bytes for r in reqs)
    server = serving.RmsdServer(db, method="tensor", query_capacity=64, hbm_budget_bytes=biggest, slots=2)
    done = server.serve(clone(reqs), realtime=False)
    assert len(done) == len(reqs)
    assert server.used == 0 and server.pool.free_rows == 64
    for r in done:
        assert np.isfinite(r.latency) and r.latency >= 0
        assert_parity(r.result.ravel(), oracle_block(db, r.queries, r.db0, r.db1).ravel(), what=f"request {r.rid}")
    s = serving.latency_summary(done)
    assert s["requests"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0


def test_serving_cancel_and_timeout(cuda):
    """Requests withdrawn or out of time finish without a result, whether it
    happens while they are queued or while their batch is on the GPU; their
    memory is returned and every other request's result is unchanged."""
    db = chain_db(2000, 300, seed=8)
    dbs = cross.FrameSet.from_frames(db)
    reqs = make_requests(db, 16, seed=9)
    alone_server = serving.RmsdServer(dbs, method="tensor", query_capacity=1024, slots=1, max_batch_requests=1)
    alone = {r.rid: r.result for r in alone_server.serve(clone(reqs), realtime=False)}

    cancel_in_flight, late_in_flight = 5, 9

    class Server(serving.RmsdServer):
        def _launch(self, slot, batch, now):
            super()._launch(slot, batch, now)
            for r in batch:
                if r.rid == cancel_in_flight:
                    r.cancel()                     # withdrawn while its batch runs
                if r.rid == late_in_flight:
                    r.timeout = now - r.arrival    # runs out while its batch runs

    server = Server(dbs, method="tensor", query_capacity=1024, slots=2, max_batch_requests=4)
    work = clone(reqs)
    work[2].cancel()                # withdrawn before it is queued
    work[7].timeout = 1e-9          # out of time while queued
    done = {r.rid: r for r in server.serve(work, realtime=False)}
    assert len(done) == len(reqs)
    want = {2: "cancelled", 7: "timed_out", cancel_in_flight: "cancelled", late_in_flight: "timed_out"}
    for rid, r in done.items():
        assert r.status == want.get(rid, "done"), (rid, r.status)
        if rid in want:
            assert r.result is None
        else:
            np.testing.assert_array_equal(r.result, alone[rid], err_msg=f"request {rid}")
    assert done[cancel_in_flight].batch >= 0 and done[late_in_flight].batch >= 0
    assert done[2].batch == -1 and done[7].batch == -1
    assert server.used == 0 and server.pool.free_rows == 1024
    s = serving.latency_summary(list(done.values()))
    assert s["requests"] == len(reqs) - len(want)
