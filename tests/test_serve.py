"""The continuous-batching server: scheduling logic on CPU against a host fake of the device
backend, and (GPU) the real thing, including alone == in-the-mix bit for bit."""
import numpy as np
import pytest

from cns_nospec_gb300 import serve as S


class FakeBox:
    """Host stand-in with the Box interface the server uses; 'bytes' = cells."""
    live = []

    def __init__(self, n, dx, cfl, eta, alam, precision=0):
        self.n, self.prec, self.steps = n, precision, 0
        FakeBox.live.append(self)

    @staticmethod
    def bytes_for(n, precision=0):
        return n[0] * n[1] * n[2]

    def init_field(self, amp, perturb, seed):
        self.seed = seed

    def sync(self):
        pass

    def health(self):
        # a request whose seed is negative stands for a solve that went non-physical
        return 4 if self.seed < 0 else 0

    def download(self):
        return np.full(1, float(self.steps))

    def close(self):
        if self in FakeBox.live:
            FakeBox.live.remove(self)


class FakeBatch:
    def __init__(self):
        self.members = []
        self.max_members = 0

    def add(self, b):
        self.members.append(b)
        self.max_members = max(self.max_members, len(self.members))

    def remove(self, b):
        self.members.remove(b)

    def advance(self, k=1):
        for b in self.members:
            b.steps += k

    def sync(self):
        pass

    def close(self):
        self.members = []


def test_request_stream_is_seeded_and_in_range():
    a = S.request_stream(rate=5.0, count=200, seed=4)
    b = S.request_stream(rate=5.0, count=200, seed=4)
    assert [(r.n, r.steps, r.precision, r.arrival) for r in a] == [(r.n, r.steps, r.precision, r.arrival) for r in b]
    assert all(24 <= r.n[0] <= 192 and 10 <= r.steps <= 200 for r in a)
    assert all(0.8 <= x <= 1.2 for r in a for x in r.amp)
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and 0.1 < np.diff(arr).mean() < 0.3
    mixed = sum(r.precision for r in a) / len(a)
    assert 0.35 < mixed < 0.65


def test_server_admits_in_order_within_budget_and_finishes_everything():
    reqs = [S.Request(i, 0.0, (10, 10, 10), steps, 0) for i, steps in enumerate([5, 3, 8, 2, 6, 4])]
    srv = S.Server(budget_bytes=2500, keep_results=True, box_cls=FakeBox, batch_cls=FakeBatch)
    rep = srv.run(reqs, realtime=False)
    assert rep["requests"] == 6
    assert rep["peak_bytes"] <= 2500
    admits = [e["admit"] for e in srv.log]
    assert admits == sorted(admits)                   # FIFO admission
    assert max(e["active"] for e in srv.log) == 2     # two 1000-cell boxes fit, a third does not
    for d in rep["done"]:
        assert d.result[0] == d.req.steps             # each box got exactly its own steps
    assert not FakeBox.live                           # every box released


def test_server_slot_limit_and_realtime_arrivals():
    reqs = [S.Request(i, 0.01 * i, (4, 4, 4), 3, i % 2) for i in range(5)]
    srv = S.Server(budget_bytes=1e9, max_active=2, box_cls=FakeBox, batch_cls=FakeBatch)
    rep = srv.run(reqs, realtime=True)
    assert rep["requests"] == 5
    assert max(e["active"] for e in srv.log) <= 2
    assert rep["latency_p99_s"] >= rep["latency_p50_s"] >= 0


def test_oversized_request_is_refused():
    reqs = [S.Request(0, 0.0, (100, 100, 100), 3, 0)]
    with pytest.raises(ValueError):
        S.Server(budget_bytes=1000, box_cls=FakeBox, batch_cls=FakeBatch).run(reqs, realtime=False)
    assert not FakeBox.live


@pytest.mark.gpu
def test_served_results_equal_alone_bitwise(gpu, cns):
    reqs = S.request_stream(rate=50.0, count=6, seed=9, nmin=16, nmax=40, smin=4, smax=12)
    budget = 2.2 * max(cns.Box.bytes_for(r.n, r.precision) for r in reqs)
    srv = S.Server(budget_bytes=budget, keep_results=True)
    rep = srv.run(reqs, realtime=False)
    assert rep["requests"] == 6
    assert max(e["active"] for e in srv.log) >= 2      # the work overlapped on the device
    assert rep["peak_bytes"] <= budget
    for d in rep["done"]:
        assert np.array_equal(d.result, S.run_alone(d.req)), d.req


def test_a_failing_solve_fails_alone():
    reqs = [S.Request(i, 0.0, (6, 6, 6), 4, 0, seed=(-1 if i == 2 else 1)) for i in range(5)]
    srv = S.Server(budget_bytes=1e9, keep_results=True, box_cls=FakeBox, batch_cls=FakeBatch)
    rep = srv.run(reqs, realtime=False)
    assert rep["requests"] == 5 and rep["failed"] == 1
    for d in rep["done"]:
        if d.req.rid == 2:
            assert d.health and d.result is None
        else:
            assert d.health == 0 and d.result[0] == 4


@pytest.mark.gpu
def test_diverging_box_does_not_disturb_its_batch(gpu, cns):
    """A box whose state goes non-physical (negative density planted at upload) is flagged;
    the boxes sharing its launches still equal their solo runs bit for bit."""
    from cns_nospec_gb300 import initdata as I
    good = [S.Request(i, 0.0, (20, 16, 24), 6, i % 2, seed=40 + i) for i in range(3)]
    batch = cns.Batch()
    boxes = []
    for r in good:
        b = cns.Box(r.n, I.box_dx(r.n), I.CFL, r.eta, r.alam, precision=r.precision)
        b.init_field(r.amp, r.perturb, r.seed)
        batch.add(b)
        boxes.append(b)
    U = I.initial_state((16, 16, 16))
    U[10, 10, 10, 0] = -1e-3
    bad = cns.Box(16, I.box_dx(16), I.CFL, I.ETA, I.ALAM)
    bad.upload(U)
    batch.add(bad)
    batch.advance(6)
    batch.sync()
    assert bad.health() != 0
    for r, b in zip(good, boxes):
        assert b.health() == 0
        assert np.array_equal(b.download(), S.run_alone(r))
    batch.close()


@pytest.mark.gpu
def test_served_results_match_the_oracle(gpu, cns, oracle):
    """Every result of a small mixed stream (FP64 and mixed requests, uneven n <= 40) against the
    reference algorithm (the oracle, cpu/advance.cpp:13-154) run on the same initial state: the
    FP64 requests within the FP64 parity bar, the mixed ones within the mixed form's bar."""
    from conftest import FP64_TOL, MIXED_TOL
    from cns_nospec_gb300 import initdata as I
    reqs = S.request_stream(rate=50.0, count=8, seed=21, nmin=16, nmax=40, smin=4, smax=12)
    assert {r.precision for r in reqs} == {cns.CNS_FP64, cns.CNS_MIXED}
    budget = 2.2 * max(cns.Box.bytes_for(r.n, r.precision) for r in reqs)
    rep = S.Server(budget_bytes=budget, keep_results=True).run(reqs, realtime=False)
    assert rep["requests"] == len(reqs) and rep["failed"] == 0
    assert rep["host_round_trips"] < rep["batch_steps"]   # several steps per round trip
    for d in rep["done"]:
        r = d.req
        b = cns.Box(r.n, I.box_dx(r.n), I.CFL, r.eta, r.alam)
        b.init_field(r.amp, r.perturb, r.seed)     # the same device-generated initial state
        U0 = b.download()
        b.close()
        ref, _ = oracle.advance(U0, r.steps, I.box_dx(r.n), I.CFL, r.eta, r.alam)
        err = I.normwise_error(d.result, ref)[0]
        assert err.max() <= (FP64_TOL if r.precision == cns.CNS_FP64 else MIXED_TOL), (r, err)
