"""GPU: the serving loop (pwmgpu_server_*): continuous batching of build and
query requests over device-resident structures under an HBM budget.  Every
answer must equal the oracle's query_support, and each request's answers in a
concurrent mix must equal the same request served alone."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GiB = 1 << 30


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def make_request(pg, rng, i):
    """The serving mix: byte Zipf texts (8 levels), DNA-like texts (3 levels),
    16-bit texts (12 levels) and 32-bit texts over 2^20 values (20 levels)."""
    kind = i % 4
    if kind == 0:
        n, L = int(rng.integers(1_000, 150_000)), 8
        text = pg.generate(pg.GEN_ZIPF256, 100 + i, n, 1)
    elif kind == 1:
        n, L = int(rng.integers(1_000, 150_000)), 3
        text = rng.choice(5, n, p=[0.29, 0.2, 0.2, 0.29, 0.02]).astype(np.uint8)
    elif kind == 2:
        n, L = int(rng.integers(1_000, 100_000)), 12
        text = rng.integers(0, 1 << L, n).astype(np.uint16)
    else:
        n, L = int(rng.integers(1_000, 60_000)), 20
        text = rng.integers(0, 1 << L, n).astype(np.uint32)
    nq = 3000
    ops = rng.integers(0, 3, nq).astype(np.uint8)
    a = np.zeros(nq, dtype=np.uint64)
    b = np.zeros(nq, dtype=np.uint64)
    counts = np.bincount(text.astype(np.int64), minlength=1 << L)
    for k in range(nq):
        if ops[k] == 0:
            a[k] = rng.integers(0, n)
        else:
            sym = int(text[rng.integers(0, n)])
            a[k] = sym
            b[k] = rng.integers(0, n + 1) if ops[k] == 1 else rng.integers(1, counts[sym] + 1)
    return dict(text=text, L=L, ops=ops, a=a, b=b)


def expected(orc, req, tree=False):
    s = orc.build(req["text"], req["L"], tree, "ps")
    q = orc.query_support(s)
    out = []
    for op, a, b in zip(req["ops"], req["a"], req["b"]):
        if op == 0:
            out.append(int(req["text"][int(a)]))
        elif op == 1:
            out.append(q.rank(int(a), int(b)))
        else:
            out.append(q.select(int(a), int(b)))
    return np.array(out, dtype=np.uint64)


@pytest.fixture(scope="module")
def mix(pg):
    _torch()
    rng = np.random.default_rng(2024)
    return [make_request(pg, rng, i) for i in range(16)]


def serve_all(pg, reqs, slots, budget=8 * GiB, tree=False):
    srv = pg.Server(budget, slots=slots)
    ids, results = [], []
    for r in reqs:
        rid, res = srv.submit(r["text"], r["L"], matrix=True, tree=tree, which=1 if tree else 0, ops=r["ops"],
                              a=r["a"], b=r["b"])
        ids.append(rid)
        results.append(res)
    infos = [srv.wait(rid) for rid in ids]
    out = [res.copy() for res in results]
    for rid in ids:
        srv.release(rid)
    stats = srv.stats()
    srv.close()
    return out, infos, stats


def test_mix_matches_oracle_and_alone(pg, orc, mix):
    mixed, infos, stats = serve_all(pg, mix, slots=4)
    # requests overlapped on the device: some started before another finished
    spans = sorted((i.start_s, i.done_s) for i in infos)
    assert any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    assert len({i.slot for i in infos}) > 1
    assert stats["completed"] == len(mix) and stats["in_use_bytes"] == 0
    for r, got in zip(mix, mixed):
        assert np.array_equal(got, expected(orc, r)), r["L"]
    # each request alone (one slot, one request at a time): identical answers
    for r, got in zip(mix, mixed):
        alone, _, _ = serve_all(pg, [r], slots=1)
        assert np.array_equal(alone[0], got)


def test_tree_queries_in_the_mix(pg, orc, mix):
    got, _, _ = serve_all(pg, mix[:6], slots=3, tree=True)
    for r, g in zip(mix[:6], got):
        assert np.array_equal(g, expected(orc, r, tree=True))


def test_admission_keeps_within_budget(pg, mix):
    # budget for about three of the larger requests: the rest wait for releases
    srv = pg.Server(160 << 20, slots=4)
    ids = []
    for r in mix:
        rid, _ = srv.submit(r["text"], r["L"], ops=r["ops"], a=r["a"], b=r["b"])
        ids.append(rid)
    done = []

    def releaser():
        for rid in ids:
            srv.wait(rid)
            done.append(rid)
            srv.release(rid)

    t = threading.Thread(target=releaser)
    t.start()
    t.join(timeout=300)
    assert not t.is_alive() and len(done) == len(ids)
    st = srv.stats()
    assert st["peak_bytes"] <= st["budget_bytes"]
    assert st["in_use_bytes"] == 0
    srv.close()


def test_request_larger_than_budget_is_refused(pg, mix):
    srv = pg.Server(1 << 20, slots=1)
    with pytest.raises(pg.PwmGpuError) as e:
        srv.submit(mix[0]["text"], mix[0]["L"])
    assert e.value.status == 2
    srv.close()


def test_query_batches_on_a_resident_structure(pg, orc, mix):
    srv = pg.Server(4 * GiB, slots=2)
    r = mix[2]
    rid, first = srv.submit(r["text"], r["L"], ops=r["ops"][:100], a=r["a"][:100], b=r["b"][:100])
    srv.wait(rid)
    exp = expected(orc, r)
    assert np.array_equal(first, exp[:100])
    qids = []
    for lo in (100, 1100, 2100):
        qid, res = srv.submit_queries(rid, r["ops"][lo:lo + 900], r["a"][lo:lo + 900], r["b"][lo:lo + 900])
        qids.append((qid, res, lo))
    for qid, res, lo in qids:
        srv.wait(qid)
        assert np.array_equal(res, exp[lo:lo + 900])
        srv.release(qid)
    srv.release(rid)
    with pytest.raises(pg.PwmGpuError):
        srv.submit_queries(rid, r["ops"][:10], r["a"][:10], r["b"][:10])
    assert srv.stats()["in_use_bytes"] == 0
    srv.close()


def test_bad_symbol_fails_only_its_request(pg, mix):
    srv = pg.Server(4 * GiB, slots=2)
    bad = np.array([1, 2, 300], dtype=np.uint16)  # 300 >= 2^8
    good = mix[0]
    rb, _ = srv.submit(bad, 8)
    rg, res = srv.submit(good["text"], good["L"], ops=good["ops"], a=good["a"], b=good["b"])
    with pytest.raises(pg.PwmGpuError) as e:
        srv.wait(rb)
    assert e.value.status == 5
    srv.wait(rg)
    assert srv.stats()["completed"] == 2
    srv.release(rb)
    srv.release(rg)
    assert srv.stats()["in_use_bytes"] == 0
    srv.close()
