"""Batched proving and a continuous-batching proof server on one GPU.

Each worker owns its own whir_ctx (CUDA stream, memory pool user, pinned staging), so proofs run by
different workers overlap on the device: one proof's host-side transcript steps and small kernels
fill the gaps of another's large kernels. Proof bytes do not depend on which worker runs a job or on
what runs beside it (every kernel is deterministic exact arithmetic and each proof owns its
transcript), which the tests check against proofs made alone.

* ``BatchProver.prove_all(jobs)`` — many independent commitments + openings of uneven sizes,
  longest jobs first over ``workers`` contexts.
* ``ProofServer`` — requests arrive over time; a request is admitted when the device-memory estimate
  of everything in flight plus its own stays under the HBM budget; admitted requests are picked up by
  the first free worker (first come, first served), so newly arrived requests join as slots and
  memory free up. Latency is completion minus arrival.
"""

import collections
import heapq
import threading
import time

import numpy as np

from . import (FIELDS, SOURCE_LIMBS, TARGET_LIMBS, Config, Context, ProtocolParameters, ProverState,
               commit_batch, multilinear_evaluate, pinned_empty)
from .inputs import Rng, field_elements

BASE_OF = {"Goldilocks1": "Goldilocks1", "Goldilocks2": "Goldilocks1", "Goldilocks3": "Goldilocks1"}


class ProofJob:
    """One commit + prove: `vectors` (batch_size x 2^nv source elements), MLE `points` with their
    `evaluations`, all host numpy arrays."""

    def __init__(self, field, nv, params, vectors, points, evaluations, session="job"):
        self.field = field
        self.nv = nv
        self.params = params
        self.vectors = np.ascontiguousarray(vectors, dtype=np.uint64)
        self.points = points
        self.evaluations = evaluations
        self.session = session
        self.narg = None
        self.hints = None
        self.arrival = None  # request arrival (host clock, set by ProofServer)
        self.start = None  # picked up by a worker
        self.done = None

    @property
    def size(self):
        return 1 << self.nv

    def memory_estimate(self):
        """Upper estimate of device bytes while the job runs: vectors, both sumcheck vectors, and
        each committed codeword with its Merkle tree (taken from the derived round schedule)."""
        cfg = Config(self.field, self.size, self.params).json()
        t = TARGET_LIMBS[FIELDS[self.field]] * 8
        s = SOURCE_LIMBS[FIELDS[self.field]] * 8
        total = self.vectors.nbytes + 2 * self.size * t
        ic = cfg["initial_committer"]
        total += ic["codeword_length"] * ic["num_cols"] * s * 2 + ic["codeword_length"] * 64
        for r in cfg["rounds"]:
            c = r["irs"]
            total += c["codeword_length"] * c["num_cols"] * t * 2 + c["codeword_length"] * 64
        return total


def make_job(field, nv, params, npoints, seed, ctx, session=None):
    """Seeded synthetic job; evaluations computed on the device (whir_multilinear_evaluate)."""
    rng = Rng(seed)
    fid = FIELDS[field]
    vec = field_elements(BASE_OF.get(field, field), params.batch_size << nv, rng=rng)
    # requests hold their vectors in page-locked memory, so commits upload them by DMA
    pinned = pinned_empty(vec.size).reshape(vec.shape)
    pinned[...] = vec
    vec = pinned
    pts = [field_elements(field, nv, rng=rng).reshape(nv, -1) for _ in range(npoints)]
    vecs = vec.reshape(params.batch_size, 1 << nv, -1)
    evals = [[multilinear_evaluate(ctx, fid, v.reshape(-1), p.reshape(-1)) for v in vecs] for p in pts]
    return ProofJob(field, nv, params, vec.reshape(params.batch_size, -1), pts, evals,
                    session or "job-%d" % seed)


def prove_job(ctx, job):
    cfg = Config(job.field, job.size, job.params)
    ps = ProverState(cfg, job.session)
    flat = job.vectors.reshape(-1)
    w = cfg.commit(ctx, ps, flat)
    cfg.prove(ctx, ps, flat, [w], job.points, [], job.evaluations)
    w.free()
    job.narg, job.hints = ps.proof()
    return job


def prove_jobs_batched(ctx, jobs):
    """Commits `jobs` (one embedding and hash engine) in shared device launches (commit_batch: one
    encode pass pair and one Merkle launch per tile step for all of them), then proves each from its
    witness. Proof bytes equal prove_job's for every job."""
    cfgs = [Config(j.field, j.size, j.params) for j in jobs]
    states = [ProverState(c, j.session) for c, j in zip(cfgs, jobs)]
    flats = [j.vectors.reshape(-1) for j in jobs]
    wits = commit_batch(ctx, cfgs, states, flats)
    for j, c, ps, flat, w in zip(jobs, cfgs, states, flats, wits):
        c.prove(ctx, ps, flat, [w], j.points, [], j.evaluations)
        w.free()
        j.narg, j.hints = ps.proof()
    return jobs


class BatchProver:
    """Proves many jobs over `workers` contexts. With batch_commit, workers take chunks of
    `commit_group` jobs of similar size, commit each chunk at once through commit_batch, then prove
    its jobs in turn; otherwise every job is committed and proved on its own."""

    def __init__(self, device=0, workers=8, batch_commit=False, commit_group=4):
        self.contexts = [Context(device) for _ in range(workers)]
        self.batch_commit = batch_commit
        self.commit_group = max(1, int(commit_group))

    def prove_all(self, jobs):
        """Proves every job; returns them in the given order (results in job.narg / job.hints)."""
        if self.batch_commit:
            return self._prove_all_batched(jobs)
        order = sorted(range(len(jobs)), key=lambda i: -jobs[i].size)
        lock = threading.Lock()
        next_idx = [0]
        errors = []

        def worker(ctx):
            while True:
                with lock:
                    if next_idx[0] >= len(order) or errors:
                        return
                    i = order[next_idx[0]]
                    next_idx[0] += 1
                try:
                    prove_job(ctx, jobs[i])
                except Exception as e:  # surfaced after all workers stop
                    with lock:
                        errors.append(e)
                    return

        threads = [threading.Thread(target=worker, args=(c,)) for c in self.contexts]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        return jobs

    def _prove_all_batched(self, jobs):
        # Groups of one embedding and hash engine, cut (largest jobs first) into chunks of
        # `commit_group` jobs of similar size: a worker commits a chunk in shared launches, then
        # proves its jobs, while other workers commit or prove theirs.
        groups = collections.defaultdict(list)
        for i, j in enumerate(jobs):
            groups[(j.field, bytes(j.params.hash_id))].append(i)
        chunks = []
        for idx in groups.values():
            idx.sort(key=lambda i: -jobs[i].size)
            chunks += [idx[k:k + self.commit_group] for k in range(0, len(idx), self.commit_group)]
        chunks.sort(key=lambda p: -sum(jobs[i].size for i in p))
        lock = threading.Lock()
        nxt = [0]
        errors = []

        def worker(ctx):
            while True:
                with lock:
                    if nxt[0] >= len(chunks) or errors:
                        return
                    part = chunks[nxt[0]]
                    nxt[0] += 1
                try:
                    prove_jobs_batched(ctx, [jobs[i] for i in part])
                except Exception as e:
                    with lock:
                        errors.append(e)
                    return

        threads = [threading.Thread(target=worker, args=(c,)) for c in self.contexts]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        return jobs

    def close(self):
        for c in self.contexts:
            c.close()


class ProofServer:
    """Continuous batching over `workers` contexts with admission by an HBM budget (bytes).

    With priority_workers > 0, that many of the workers own contexts with raised stream priority and
    take the oldest admitted request of fewer than 2^large_nv coefficients first (priority_large:
    of at least 2^large_nv); the other workers take the oldest request of the other class first.
    Either falls back to the oldest request of any size. The kernels of the favoured class then go
    ahead of the pending blocks of the other's.

    With max_work set, a request starts only while the coefficients (batch_size x 2^nv) of the
    requests in service plus its own stay within max_work, or when none is in service; a worker
    whose pick (the oldest request, or with priority workers the oldest of its class) does not fit
    waits rather than taking a later one. Fewer large requests then share the device at once, so
    each runs closer to its time alone, at the cost of more queueing."""

    def __init__(self, device=0, workers=8, hbm_budget=150 << 30, priority_workers=0, large_nv=22,
                 priority_large=False, max_work=None):
        priority_workers = max(0, min(priority_workers, workers))
        self.contexts = [Context(device, priority=1) for _ in range(priority_workers)]
        self.contexts += [Context(device) for _ in range(workers - priority_workers)]
        favoured = bool(priority_large)
        self.prefers_large = [favoured] * priority_workers + [not favoured] * (workers - priority_workers)
        self.large_nv = large_nv
        self.split = priority_workers > 0
        self.budget = hbm_budget
        self.max_work = max_work

    def run(self, jobs, arrivals):
        """Replays a request trace: job i arrives `arrivals[i]` seconds after the start. Returns
        per-job latencies in seconds (completion - arrival) in job order; each job also keeps its
        arrival, start (picked up by a worker) and completion times, so latency splits into queueing
        (start - arrival) and service (done - start)."""
        n = len(jobs)
        est = [j.memory_estimate() for j in jobs]
        if any(e > self.budget for e in est):
            raise ValueError("a request exceeds the HBM budget on its own")
        work = [j.vectors.shape[0] << j.nv for j in jobs]
        cv = threading.Condition()
        pending = collections.deque()  # arrived, not yet admitted (FIFO)
        admitted = collections.deque()  # admitted, waiting for a worker
        state = {"in_use": 0, "taken": 0, "work": 0, "error": None}
        t0 = time.perf_counter()

        def admit_locked():
            while pending and state["in_use"] + est[pending[0]] <= self.budget:
                i = pending.popleft()
                state["in_use"] += est[i]
                admitted.append(i)

        def feeder():
            for i in sorted(range(n), key=lambda k: arrivals[k]):
                delay = t0 + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                with cv:
                    jobs[i].arrival = time.perf_counter()
                    pending.append(i)
                    admit_locked()
                    cv.notify_all()

        def pick_locked(large):
            # position of the oldest admitted request of the preferred size class, else of the oldest
            # of any; None while the work cap holds it back
            k = 0
            if self.split:
                k = next((q for q, i in enumerate(admitted) if (jobs[i].nv >= self.large_nv) == large), 0)
            i = admitted[k]
            if self.max_work is not None and state["work"] > 0 and state["work"] + work[i] > self.max_work:
                return None
            return k

        def worker(ctx, large):
            while True:
                with cv:
                    while True:
                        if state["error"] is not None:
                            return  # failed elsewhere
                        if admitted:
                            k = pick_locked(large)
                            if k is not None:
                                break
                        elif state["taken"] >= n:
                            return  # every job has been taken
                        cv.wait(timeout=0.05)
                    i = admitted[k]
                    del admitted[k]
                    state["taken"] += 1
                    state["work"] += work[i]
                    jobs[i].start = time.perf_counter()
                try:
                    prove_job(ctx, jobs[i])
                except Exception as e:
                    with cv:
                        state["error"] = e
                        cv.notify_all()
                    return
                with cv:
                    jobs[i].done = time.perf_counter()
                    state["in_use"] -= est[i]
                    state["work"] -= work[i]
                    admit_locked()
                    cv.notify_all()

        threads = [threading.Thread(target=feeder)] + [threading.Thread(target=worker, args=(c, lg))
                                                       for c, lg in zip(self.contexts, self.prefers_large)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if state["error"] is not None:
            raise state["error"]
        return [jobs[i].done - jobs[i].arrival for i in range(n)]

    def close(self):
        for c in self.contexts:
            c.close()


def batched_workload(ctx, count=64, seed=4, sizes=(14, 16, 18, 20, 22)):
    """Batched commit + open workload: `count` independent Goldilocks3 polynomials with d drawn
    uniformly from `sizes`, Blake3, rate 1/2, folding factor 4, 1-2 evaluation points each."""
    r = Rng(seed)
    params = ProtocolParameters(unique_decoding=False, security_level=128, pow_bits=20, starting_log_inv_rate=1,
                                initial_folding_factor=4, folding_factor=4, hash_id="Blake3")
    jobs = []
    for k in range(count):
        d = sizes[int(r.raw(1)[0] % len(sizes))]
        npts = 1 + int(r.raw(1)[0] % 2)
        jobs.append(make_job("Goldilocks3", d, params, npts, seed * 1000 + k, ctx, session="batch-%d" % k))
    return jobs


def serving_workload(ctx, count=48, seed=5, sizes=(16, 18, 20, 22, 24)):
    """Serving trace jobs: Goldilocks2 / Blake3, folding factor 4, rate 1/2 or 1/4, 1-4 points,
    d log-uniform over `sizes` (uniform over the exponent list), unique decoding."""
    r = Rng(seed)
    jobs = []
    for k in range(count):
        d = sizes[int(r.raw(1)[0] % len(sizes))]
        rate = 1 + int(r.raw(1)[0] % 2)
        npts = 1 + int(r.raw(1)[0] % 4)
        params = ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20, starting_log_inv_rate=rate,
                                    initial_folding_factor=4, folding_factor=4, hash_id="Blake3")
        jobs.append(make_job("Goldilocks2", d, params, npts, seed * 1000 + k, ctx, session="serve-%d" % k))
    return jobs


def poisson_arrivals(count, rate_per_s, seed=6):
    """Arrival times (seconds) of a Poisson process with the given rate."""
    gaps = np.random.default_rng(seed).exponential(1.0 / rate_per_s, size=count)
    return list(np.cumsum(gaps) - gaps[0])
