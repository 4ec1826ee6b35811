"""Benchmark of the WHIR prover path on GB300.

Workload (the reference's headline configuration on one GPU): WHIR PCS commit + prove, d = 24
(2^24 uniform random Goldilocks coefficients, codeword 2^25 elements), Basefield<Field64_2>
(Goldilocks2), Blake3 Merkle trees, log_inv_rate 1, folding factor 4, security 100, unique decoding,
pow_bits 20, one uniform random evaluation point. Inputs are seeded synthetic data (SplitMix64,
whir_gb300/inputs.py). The metric is milliseconds per proof (commit + prove, as the reference's
benchmark.rs:238-258 times it); lower is better.

One step = one full proof. `value` times steps with the polynomial already resident in HBM;
`e2e` times the same proofs through the public C ABI from pinned host memory (the host->device
copy of the coefficients and every device->host read of the proof happen inside the timed region).
Every proof's working set (>1 GiB) exceeds L2 (129 MB), and an L2-sized buffer is also rewritten
between steps.

--impl reference runs the reference's CPU algorithm (the repository's C++ restatement in oracle/,
since the Rust reference cannot be built here) on all host cores for the same workload.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from whir_gb300.replicas import max_over_ranks  # noqa: E402

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# DRAM traffic / algorithmic bytes of a kernel family, from one ncu capture (profiles/
# ncu_encode_kernels_prove_d24_goldilocks2.md): the initial commitment's encode_cols + encode_rows
# moved 350.8 + 549.7 MB of DRAM for 402,653,184 algorithmic bytes. The encode kernels' traffic grows
# in proportion to the elements they process, so per-launch traffic = algorithmic bytes x this ratio.
NCU_TRAFFIC_RATIO = {"encode": (134.601472e6 + 216.216576e6 + 268.512768e6 + 281.217536e6) / 402653184.0}

# The encode kernels are bound by the integer ALU pipe, not HBM. Warp instructions that the commitment
# encodes of one d=24 proof of this workload issue to the ALU pipe (ncu sm__inst_executed_pipe_alu.sum
# over the nine encode_cols / encode_rows launches of the four commitments; profiles/
# ncu_encode_alu_prove_d24_goldilocks2.md), and that pipe's peak issue rate per SM and cycle
# (sm__inst_executed_pipe_alu.avg.peak_sustained). The count depends on the code and the shapes only,
# not on the data, so achieved = count / live encode time.
ENCODE_ALU_WARP_INST = {24: 924550784}
ALU_PEAK_WARP_INST_PER_SM_CYCLE = 2.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nv", type=int, default=24)
    ap.add_argument("--cpu-nv", type=int, default=None,
                    help="d of the CPU-baseline proofs (default: --nv, the measured workload itself)")
    ap.add_argument("--cpu-runs", type=int, default=5, help="timed CPU-baseline proofs (after one warm-up)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default encode plans and Merkle tiles")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched / serving measurements")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--serve-jobs", type=int, default=96, help="distinct requests of the serving trace")
    ap.add_argument("--serve-repeat", type=int, default=3,
                    help="times the trace replays the distinct requests (arrival order stays Poisson)")
    ap.add_argument("--workers", type=int, default=8,
                    help="worker contexts for the batched / serving runs (8: 914 proofs/s vs 755 with 4)")
    ap.add_argument("--multilimb-nv", type=int, default=20)
    ap.add_argument("--no-multilimb", action="store_true", help="skip the Field256 / Field192 measurement")
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend="gloo")
    return rank, world, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(nv):
    import whir_gb300 as W
    from whir_gb300.inputs import Rng, field_elements
    params = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20, starting_log_inv_rate=1,
                                  initial_folding_factor=4, folding_factor=4, hash_id="Blake3")
    rng = Rng(2)  # seed = config index
    vec = rng.goldilocks(1 << nv)
    point = field_elements("Goldilocks2", nv, rng=rng).reshape(nv, 2)
    return params, vec, point


def evaluation(ctx, vec, point):
    import whir_gb300 as W
    return W.multilinear_evaluate(ctx, W.GOLDILOCKS2, vec, point.reshape(-1))


def batched_and_serving(args, dev):
    """Batched workload (64 Goldilocks3 polynomials, d in {14..22}) proved back to
    back on one context and batched over several contexts, then a Poisson serving trace of Goldilocks2
    requests (d in {16..24}) at 70% of the measured batched capacity. Host wall clock (several streams
    run at once); every batched / served proof is checked byte-identical to the back-to-back one."""
    import whir_gb300 as W
    from whir_gb300 import serving
    ctx = W.Context(dev)
    out = {}
    jobs = serving.batched_workload(ctx, count=args.batch_jobs)

    def median_pass_s(prover, js, passes=3):
        # Host wall clock of whole passes over the jobs; the median of three damps the shared host's
        # load swings (these small proofs are bound by host round trips).
        ts = []
        for _ in range(passes):
            t0 = time.perf_counter()
            prover.prove_all(js)
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)), ts

    one = serving.BatchProver(dev, workers=1)
    one.prove_all(jobs[:4])  # warm-up
    plain_s, _ = median_pass_s(one, jobs)
    ref = [(j.narg, j.hints) for j in jobs]
    one.close()
    many = serving.BatchProver(dev, workers=args.workers)
    many.prove_all(jobs[:8])
    batch_s, batch_passes = median_pass_s(many, jobs)
    many.close()
    same = all((j.narg, j.hints) == r for j, r in zip(jobs, ref))
    # Batched commits: each worker commits its share of the jobs in shared launches (one encode pass
    # pair and one Merkle launch per tile step over a job table), then proves them.
    bc = serving.BatchProver(dev, workers=args.workers, batch_commit=True)
    bc.prove_all(jobs[:8])
    bc_s, bc_passes = median_pass_s(bc, jobs)
    bc.close()
    same_bc = all((j.narg, j.hints) == r for j, r in zip(jobs, ref))
    out["batched"] = {
        "workload": "%d x WHIR commit+prove, Goldilocks3, d in {14,16,18,20,22}, Blake3, rate 1/2, k=4, sec 128 "
                    "list decoding, 1-2 points" % len(jobs),
        "proofs_per_s": len(jobs) / batch_s, "back_to_back_proofs_per_s": len(jobs) / plain_s,
        "speedup_vs_back_to_back": plain_s / batch_s, "workers": args.workers,
        "bit_exact_vs_plain": same and same_bc,
        "passes_proofs_per_s": [len(jobs) / t for t in batch_passes],
        "batched_commit_proofs_per_s": len(jobs) / bc_s,
        "batched_commit_passes_proofs_per_s": [len(jobs) / t for t in bc_passes],
        "timing": "host wall clock, median of 3 passes"}
    sjobs = serving.serving_workload(ctx, count=args.serve_jobs)
    # The trace replays the distinct requests `serve_repeat` times (the copies share the page-locked
    # vectors), so its percentiles rest on more requests than there are distinct inputs.
    trace = [serving.ProofJob(j.field, j.nv, j.params, j.vectors, j.points, j.evaluations, j.session)
             for _ in range(max(1, args.serve_repeat)) for j in sjobs]
    cap = serving.BatchProver(dev, workers=args.workers)
    cap.prove_all(sjobs)  # warm-up, and the reference proofs
    sref = [(j.narg, j.hints) for j in sjobs]
    cap.close()
    # The server's own capacity: every request of the trace queued at once and served first come
    # first served (median of three runs). Batched passes, longest job first, ran 40 % above what the
    # server sustains in arrival order, so 70 % of their rate overloaded it.
    srv = serving.ProofServer(dev, workers=args.workers, hbm_budget=150 << 30)
    runs = []
    for _ in range(3):
        t0 = time.perf_counter()
        srv.run(trace, [0.0] * len(trace))
        runs.append(time.perf_counter() - t0)
    srv.close()
    capacity = len(trace) / float(np.median(runs))
    rate = 0.7 * capacity
    arrivals = serving.poisson_arrivals(len(trace), rate, seed=6)

    def serve(**policy):
        srv = serving.ProofServer(dev, workers=args.workers, hbm_budget=150 << 30, large_nv=22, **policy)
        t = time.perf_counter()
        lat = srv.run(trace, arrivals)
        wall = time.perf_counter() - t
        srv.close()
        queue = [j.start - j.arrival for j in trace]
        service = [j.done - j.start for j in trace]
        p99_by_d = {}
        for d in sorted({j.nv for j in trace}):
            ls = [x for x, j in zip(lat, trace) if j.nv == d]
            p99_by_d[str(d)] = float(np.percentile(ls, 99)) * 1e3
        return {
            "p50_ms": float(np.percentile(lat, 50)) * 1e3, "p99_ms": float(np.percentile(lat, 99)) * 1e3,
            "queue_p50_ms": float(np.percentile(queue, 50)) * 1e3, "queue_p99_ms": float(np.percentile(queue, 99)) * 1e3,
            "service_p50_ms": float(np.percentile(service, 50)) * 1e3,
            "service_p99_ms": float(np.percentile(service, 99)) * 1e3,
            "p99_by_d_ms": p99_by_d, "proofs_per_s": len(trace) / wall,
            "bit_exact_vs_plain": all((j.narg, j.hints) == sref[k % len(sjobs)] for k, j in enumerate(trace))}

    fifo = serve()
    others = [(serve(priority_workers=2), "2 of the workers on raised-priority streams take requests of d < 22 "
                                          "first, the others larger ones first"),
              (serve(max_work=2 << 24), "first come first served, a request starting only while the requests in "
                                        "service hold at most 2 x 2^24 coefficients with it (or none is in service)")]
    ctx.close()
    out["serving"] = {
        "workload": "%d requests (%d distinct, each replayed %d times), Goldilocks2 Blake3 k=4, d uniform over "
                    "{16,18,20,22,24}, rate 1/2 or 1/4, 1-4 points, unique decoding; Poisson arrivals at 70%% of "
                    "the server's capacity (median of three runs with the whole trace queued at once); 150 GB HBM "
                    "budget; request vectors in page-locked memory"
                    % (len(trace), len(sjobs), max(1, args.serve_repeat)),
        "capacity_proofs_per_s": capacity, "arrival_rate_per_s": rate, **fifo, "workers": args.workers,
        "policy": "first come first served",
        "other_policies": [{**r, "policy": name} for r, name in others],
        "timing": "host wall clock, the same arrival trace for every policy"}
    return out


def multilimb(args, dev):
    """Multi-limb workload: WHIR PCS commit+prove at d=20 over Field256 then Field192 (Montgomery form),
    SHA3 Merkle trees, rate 1/4, k=4, security 128 list decoding, pow 20, 4 uniform random evaluation
    points. Device-resident input, CUDA events on the context's stream; proof bytes checked identical
    across steps. The CPU column times the oracle prover on the same input (one proof per field)."""
    import torch

    import whir_gb300 as W
    from whir_gb300.inputs import Rng, field_elements
    nv = args.multilimb_nv
    ctx = W.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)
    params = W.ProtocolParameters(unique_decoding=False, security_level=128, pow_bits=20, starting_log_inv_rate=2,
                                  initial_folding_factor=4, folding_factor=4, hash_id="Sha3")
    out = {"workload": "WHIR PCS commit+prove d=%d, SHA3, rate 1/4, k=4, sec 128 list decoding, pow 20, 4 points"
                       % nv}
    for field in ("Field256", "Field192"):
        fid = W.FIELDS[field]
        r = Rng(fid * 20)
        vec = field_elements(field, 1 << nv, rng=r).reshape(-1)
        pts = [field_elements(field, nv, rng=r).reshape(-1) for _ in range(4)]
        evs = [[W.multilinear_evaluate(ctx, fid, vec, p)] for p in pts]
        cfg = W.Config(field, 1 << nv, params)
        d_vec = ctx.alloc(vec.nbytes)
        ctx.upload(d_vec, vec)

        def one():
            ps = W.ProverState(cfg, "bench " + field)
            w = cfg.commit(ctx, ps, d_vec, on_device=True)
            cfg.prove(ctx, ps, d_vec, [w], pts, [], evs, on_device=True)
            w.free()
            return ps.proof()

        ref = None
        for _ in range(2):
            ref = one()
        ctx.set_profiling(True)
        times = []
        for _ in range(max(3, args.steps // 2)):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            got = one()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            assert got == ref, "proof bytes changed between runs"
        prof = ctx.profile()
        ctx.set_profiling(False)
        ctx.free(d_vec)
        entry = {"prove_ms": float(np.mean(times)), "p50_ms": float(np.percentile(times, 50)),
                 "kernel_families_ms_per_proof": {k: v[0] / len(times) for k, v in prof.items() if v[1]},
                 "narg_bytes": len(ref[0]), "hint_bytes": len(ref[1])}
        if not args.no_cpu_baseline:
            import oracle
            op = oracle.make_params(unique_decoding=False, security_level=128, pow_bits=20, starting_log_inv_rate=2,
                                    hash_id=oracle.ENGINE_SHA3)
            vv = vec.reshape(1, 1 << nv, -1)
            pp = [p.reshape(nv, -1) for p in pts]
            t0 = time.perf_counter()
            pr = oracle.whir_prove(fid, op, nv, "bench " + field, vv, pp, [], evs)
            sec = time.perf_counter() - t0
            entry["cpu_baseline"] = {"value": sec * 1e3, "unit": "ms", "cores": oracle.lib().oracle_num_threads(),
                                     "kind": "port", "sample": "1 proof, same input"}
            entry["bit_exact_vs_cpu"] = (pr.narg, pr.hints) == ref
        out[field] = entry
    ctx.close()
    return out


def algorithmic_bytes(cfg_json, nv):
    """Per-proof algorithmic HBM bytes of each kernel family (input + output of each pass)."""
    s_elem, t_elem = 8, 16
    enc = 0
    ic = cfg_json["initial_committer"]
    enc += ic["vector_size"] * ic["num_vectors"] * s_elem + ic["codeword_length"] * ic["num_cols"] * s_elem
    for r in cfg_json["rounds"]:
        c = r["irs"]
        enc += c["vector_size"] * t_elem + c["codeword_length"] * c["num_cols"] * t_elem
    sc = 0
    sizes = [(cfg_json["initial_sumcheck"]["initial_size"], cfg_json["initial_sumcheck"]["num_rounds"])]
    sizes += [(r["sumcheck"]["initial_size"], r["sumcheck"]["num_rounds"]) for r in cfg_json["rounds"]]
    for n, rounds in sizes:
        for k in range(rounds):
            m = n >> k
            sc += 2 * m * t_elem + (m * t_elem if k > 0 else 0)  # read a, b (+ write halves when folding)
        sc += 2 * (n >> rounds) * t_elem * 2  # final fold of a and b
    lift = (1 << nv) * (s_elem + t_elem)
    eq = (1 << nv) * t_elem * 2  # read-modify-write of the covector
    return {"encode": enc, "sumcheck": sc, "lift": lift, "eq": eq}


def hbm_peak():
    try:
        d = json.load(open(MEASURED_PEAKS))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def cpu_workload(nv):
    """The measured workload's inputs for the oracle: the same seeded coefficients and point as
    `workload(nv)`, and the statement's evaluation computed on the CPU."""
    import oracle
    from whir_gb300.inputs import Rng, field_elements
    rng = Rng(2)
    vec = rng.goldilocks(1 << nv)
    point = field_elements("Goldilocks2", nv, rng=rng).reshape(nv, 2)
    ev = oracle.multilinear_extend(oracle.GOLDILOCKS2, vec, point.reshape(-1))
    op = oracle.make_params(unique_decoding=True, security_level=100, pow_bits=20)
    return op, vec, point, ev


def cpu_prove(nv, op, vec, point, ev):
    """One commit + prove of the oracle prover (the reference algorithm restated in C++, on every
    host core). Returns (seconds, proof)."""
    import oracle
    t0 = time.perf_counter()
    pr = oracle.whir_prove(oracle.GOLDILOCKS2, op, nv, "bench", vec.reshape(1, -1), [point], [], [[ev]])
    return time.perf_counter() - t0, pr


def cpu_baseline(args):
    """Times the oracle prover on the measured workload itself (d = --cpu-nv, default --nv): one
    warm-up proof, then --cpu-runs timed proofs; the value is their median. Also returns the first
    proof's bytes so the GPU proof can be compared with it."""
    import oracle
    nv = args.cpu_nv if args.cpu_nv is not None else args.nv
    op, vec, point, ev = cpu_workload(nv)
    _, pr = cpu_prove(nv, op, vec, point, ev)
    secs = [cpu_prove(nv, op, vec, point, ev)[0] for _ in range(max(1, args.cpu_runs))]
    line = {"value": float(np.median(secs)) * 1e3, "unit": "ms", "cores": oracle.lib().oracle_num_threads(),
            "kind": "port", "mean_ms": float(np.mean(secs)) * 1e3, "runs_ms": [t * 1e3 for t in secs],
            "sample": "%d proof(s) at d=%d after 1 warm-up, median (the measured workload itself, no scaling)"
                      % (len(secs), nv)}
    return line, (pr.narg, pr.hints), nv


def run_reference(args):
    """The reference arm: the oracle prover (the reference's CPU algorithm, restated in C++) on all
    host cores, one proof of the measured workload per step, --warmup untimed proofs first."""
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    import oracle
    nv = args.nv
    op, vec, point, ev = cpu_workload(nv)
    for _ in range(args.warmup):
        cpu_prove(nv, op, vec, point, ev)
    secs = [cpu_prove(nv, op, vec, point, ev)[0] for _ in range(args.steps)]
    ms = float(np.median(secs)) * 1e3
    cores = oracle.lib().oracle_num_threads()
    line = {
        "impl": "reference", "metric": "prove_ms_d%d_goldilocks2_blake3" % nv, "value": ms, "unit": "ms",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(secs)) * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks field)",
        "data": "synthetic (SplitMix64 seed 2, uniform field elements)",
        "config": {"workload": "WHIR PCS commit+prove d=%d Goldilocks2 Blake3 rate 1/2 k=4 sec 100 UD pow 20, 1 point"
                               % nv, "statistic": "value = median of the steps, ms_per_step = their mean"},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port",
                         "sample": "each step: 1 proof at d=%d (the measured workload itself, no scaling)" % nv},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch

    import whir_gb300 as W
    rank, world, local, dist = dist_setup(args.gpus)
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    nv = args.nv
    params, vec, point = workload(nv)
    ctx = W.Context(dev)
    ev = evaluation(ctx, vec, point)
    cfg = W.Config("Goldilocks2", 1 << nv, params)
    cfg_json = cfg.json()
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:%d" % dev)

    # Resident input for `value`.
    d_vec = ctx.alloc(vec.nbytes)
    ctx.upload(d_vec, vec)

    def one_proof(on_device, src):
        ps = W.ProverState(cfg, "bench")
        w = cfg.commit(ctx, ps, src, on_device=on_device)
        cfg.prove(ctx, ps, src, [w], [point], [], [[ev]], on_device=on_device)
        w.free()
        return ps

    tuned = None
    if not args.no_autotune:
        # Encode plans and Merkle tile heights measured for this configuration's commitment shapes
        # (whir_autotune); proofs are bit-identical under any choice.
        rep = W.autotune(ctx, cfg, reps=3)
        tuned = [{"shape": [s["n_msgs"], s["msg_len"], s["codeword_len"], s["elem_bytes"]], "pick": s["pick"],
                  "pick_ms": s["pick_ms"], "default_ms": s["default_ms"], "merkle_tile_log": s["merkle_pick"]}
                 for s in rep["shapes"]]
    ref_narg = None
    for _ in range(args.warmup):
        ps = one_proof(True, d_vec)
        ref_narg = ps.proof()
    barrier(dist)
    torch.cuda.synchronize()

    times = []
    first_timed_proof = None
    launches0 = ctx.launch_count()
    sampler = ClockSampler(dev)
    sampler.start()
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ps = one_proof(True, d_vec)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        proof = ps.proof()
        assert proof == ref_narg, "proof bytes changed between runs"
        if first_timed_proof is None:
            first_timed_proof = proof
    clocks = sampler.stop()
    launches = ctx.launch_count() - launches0
    # Per-family device time (CUDA events around each kernel family on the context's stream), taken
    # in separate untimed proofs so the event records do not perturb the timed ones.
    prof_steps = max(3, args.steps // 2)
    ctx.set_profiling(True)
    for _ in range(prof_steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        one_proof(True, d_vec)
    prof = ctx.profile()
    ctx.set_profiling(False)
    barrier(dist)
    torch.cuda.synchronize()
    total_ms = max_over_ranks(dist, float(np.sum(times)))
    ms_per_proof_job = total_ms / (args.steps * world)

    # End to end through the public API from pinned host memory.
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty(vec.size, dtype=torch.int64).pin_memory()
        host = pinned.numpy().view(np.uint64)
        host[:] = vec
        for _ in range(max(1, args.warmup // 2)):
            one_proof(False, host)
        h0, d0 = ctx.transfer_bytes()
        et = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ps = one_proof(False, host)
            e1.record(stream)
            e1.synchronize()
            et.append(e0.elapsed_time(e1))
        h1, d1 = ctx.transfer_bytes()
        e2e_total = max_over_ranks(dist, float(np.sum(et)))
        e2e = {"value": e2e_total / (args.steps * world), "unit": "ms",
               "h2d_bytes_per_step": int((h1 - h0) / args.steps), "d2h_bytes_per_step": int((d1 - d0) / args.steps)}

    if rank != 0:
        return
    # Roofline of the dominant kernel family, timed live with CUDA events on the context's stream.
    alg = algorithmic_bytes(cfg_json, nv)
    fam = max((f for f in prof if prof[f][1] > 0), key=lambda f: prof[f][0])
    ms_f, calls_f = prof[fam]
    peak, peak_kind = hbm_peak()
    roofline = None
    if fam in alg:
        per_call_bytes = alg[fam] * prof_steps / calls_f
        achieved = per_call_bytes / (ms_f / calls_f * 1e-3) / 1e9
        ratio = NCU_TRAFFIC_RATIO.get(fam)
        roofline = {"bound": "hbm", "kernel_family": fam, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": peak_kind,
                    "traffic": per_call_bytes * ratio if ratio else None,
                    "algorithmic_bytes_per_launch": per_call_bytes, "avg_launch_ms": ms_f / calls_f}
    else:
        roofline = {"bound": "integer", "kernel_family": fam, "achieved": None, "peak": peak, "unit": "GB/s",
                    "frac": None, "traffic": None, "avg_launch_ms": ms_f / calls_f}
    # The bound that sets the encode kernels' time: ALU-pipe issue rate at the SM clock sampled during the
    # timed region.
    roofline_alu = None
    if nv in ENCODE_ALU_WARP_INST and prof.get("encode", (0, 0))[1]:
        ms_e = prof["encode"][0] / prof_steps
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
        if mhz:
            ach = ENCODE_ALU_WARP_INST[nv] / (ms_e * 1e-3) / 1e9
            pk = sms * ALU_PEAK_WARP_INST_PER_SM_CYCLE * mhz * 1e6 / 1e9
            roofline_alu = {"bound": "alu", "kernel_family": "encode", "achieved": ach, "peak": pk,
                            "unit": "G warp-inst/s", "frac": ach / pk,
                            "alu_warp_inst_per_proof": ENCODE_ALU_WARP_INST[nv], "encode_ms_per_proof": ms_e,
                            "count_source": "ncu count of one proof under the default encode plans",
                            "peak_source": "%d SMs x %.1f ALU warp-inst/cycle x %.0f MHz sampled SM clock"
                                           % (sms, ALU_PEAK_WARP_INST_PER_SM_CYCLE, mhz)}
    cpu, bit_exact = None, None
    if not args.no_cpu_baseline:
        cpu, cpu_proof, cpu_nv = cpu_baseline(args)
        bit_exact = (cpu_proof == first_timed_proof) if cpu_nv == nv else None
    extra = {} if args.no_batch else batched_and_serving(args, dev)
    if not args.no_multilimb:
        extra["multilimb"] = multilimb(args, dev)
    line = {
        "metric": "prove_ms_d%d_goldilocks2_blake3" % nv, "value": ms_per_proof_job, "unit": "ms",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks field)",
        "data": "synthetic (SplitMix64 seed 2, uniform field elements)",
        "config": {"workload": "WHIR PCS commit+prove d=%d Goldilocks2 Blake3 rate 1/2 k=4 sec 100 UD pow 20, 1 point"
                               % nv, "parallelism": "replicas x%d" % world,
                   "l2": "working set > L2 and a 256 MiB buffer rewritten between steps",
                   "p50_ms": float(np.percentile(times, 50)), "p99_ms": float(np.percentile(times, 99))},
        "roofline": roofline,
        "roofline_alu": roofline_alu,
        "kernel_families_ms_per_proof": {k: v[0] / prof_steps for k, v in prof.items() if v[1]},
        "autotune": tuned,
        "cpu_baseline": cpu,
        "bit_exact_vs_cpu": bit_exact,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        **extra,
    }
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
