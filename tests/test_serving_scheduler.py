"""Host-side scheduling of serving.ProofServer, run on CPU with stand-ins for the device context and the
prover: every request is served once, admission keeps the HBM budget, the work cap bounds what is in
service at once, and priority workers take their size class first."""

import threading
import time

import pytest

from whir_gb300 import serving


class FakeContext:
    def __init__(self, device=0, priority=0):
        self.priority = priority

    def close(self):
        pass


class FakeVectors:
    def __init__(self, batch):
        self.shape = (batch,)


class FakeJob:
    def __init__(self, nv, mem=1, batch=1):
        self.nv = nv
        self.vectors = FakeVectors(batch)
        self.mem = mem
        self.arrival = self.start = self.done = None
        self.ctx = None

    def memory_estimate(self):
        return self.mem


class Recorder:
    """prove_job stand-in: sleeps in proportion to the request's size and records what was in service."""

    def __init__(self, scale=0.0005):
        self.scale = scale  # seconds of sleep for a 2^10-coefficient request
        self.lock = threading.Lock()
        self.running = []
        self.max_work_seen = []
        self.max_mem_seen = 0

    def __call__(self, ctx, job):
        with self.lock:
            self.running.append(job)
            work = sum(j.vectors.shape[0] << j.nv for j in self.running)
            self.max_work_seen.append((len(self.running), work))
            self.max_mem_seen = max(self.max_mem_seen, sum(j.mem for j in self.running))
        job.ctx = ctx
        time.sleep(self.scale * (1 << (job.nv - 10)))
        with self.lock:
            self.running.remove(job)
        return job


@pytest.fixture
def fake(monkeypatch):
    rec = Recorder()
    monkeypatch.setattr(serving, "Context", FakeContext)
    monkeypatch.setattr(serving, "prove_job", rec)
    return rec


def _jobs(n, sizes=(10, 11, 12, 13, 14), mem=1):
    return [FakeJob(sizes[(7 * k) % len(sizes)], mem=mem) for k in range(n)]


def _arrivals(n, gap=0.0004):
    return [k * gap for k in range(n)]


@pytest.mark.parametrize("kw", [dict(workers=4), dict(workers=4, priority_workers=2),
                                dict(workers=4, priority_workers=2, priority_large=True),
                                dict(workers=4, max_work=3 << 13), dict(workers=1)])
def test_every_request_served_once(fake, kw):
    jobs = _jobs(30)
    srv = serving.ProofServer(hbm_budget=1 << 40, large_nv=13, **kw)
    lat = srv.run(jobs, _arrivals(len(jobs)))
    srv.close()
    assert len(lat) == len(jobs) and all(x > 0 for x in lat)
    for j in jobs:
        assert j.arrival <= j.start <= j.done


def test_hbm_budget_bounds_requests_in_service(fake):
    jobs = _jobs(24, mem=10)
    srv = serving.ProofServer(workers=6, hbm_budget=25)
    srv.run(jobs, [0.0] * len(jobs))
    srv.close()
    assert fake.max_mem_seen <= 25


def test_work_cap_bounds_requests_in_service(fake):
    cap = 3 << 13
    jobs = _jobs(40)
    srv = serving.ProofServer(workers=6, hbm_budget=1 << 40, max_work=cap)
    srv.run(jobs, [0.0] * len(jobs))
    srv.close()
    # over the cap only when a single request is in service on its own
    assert all(work <= cap or count == 1 for count, work in fake.max_work_seen)
    # strictly oldest first under the cap
    starts = sorted(range(len(jobs)), key=lambda i: jobs[i].start)
    assert starts == list(range(len(jobs)))


def test_request_over_cap_runs_alone(fake):
    jobs = [FakeJob(10), FakeJob(15), FakeJob(10)]
    srv = serving.ProofServer(workers=3, hbm_budget=1 << 40, max_work=1 << 12)
    srv.run(jobs, [0.0, 0.0, 0.0])
    srv.close()
    # the 2^15 request neither joins the first nor lets the third overtake it
    assert all(count == 1 for count, _ in fake.max_work_seen)
    assert jobs[0].done <= jobs[1].start and jobs[1].done <= jobs[2].start


@pytest.mark.parametrize("large", [False, True])
def test_priority_workers_take_their_class_first(fake, large):
    # Two long requests hold both workers while two small and two large ones queue up; the priority
    # worker's next request is then the oldest of its class. Slow stand-in proofs (the large ones take
    # 32 ms) keep the outcome clear of thread-scheduling jitter.
    fake.scale = 0.002
    jobs = [FakeJob(16), FakeJob(16), FakeJob(10), FakeJob(14), FakeJob(10), FakeJob(14)]
    srv = serving.ProofServer(workers=2, hbm_budget=1 << 40, priority_workers=1, large_nv=12,
                              priority_large=large)
    prio = srv.contexts[0]
    assert prio.priority == 1 and srv.contexts[1].priority == 0
    srv.run(jobs, [0.0, 0.0, 0.005, 0.005, 0.005, 0.005])
    srv.close()
    assert jobs[0].ctx is not jobs[1].ctx
    later = sorted((j for j in jobs[2:] if j.ctx is prio), key=lambda j: j.start)
    assert later and (later[0].nv >= 12) == large


def test_server_rejects_request_over_budget_on_cpu(fake):
    srv = serving.ProofServer(workers=1, hbm_budget=5)
    with pytest.raises(ValueError):
        srv.run([FakeJob(10, mem=6)], [0.0])
    srv.close()


def test_prover_error_surfaces(fake, monkeypatch):
    def boom(ctx, job):
        raise RuntimeError("prover failed")

    monkeypatch.setattr(serving, "prove_job", boom)
    srv = serving.ProofServer(workers=2, hbm_budget=1 << 40)
    with pytest.raises(RuntimeError, match="prover failed"):
        srv.run(_jobs(5), _arrivals(5))
    srv.close()
