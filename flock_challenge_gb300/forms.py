"""Batched and served proving measured against the plain GPU path.

python -m flock_challenge_gb300.forms [--batch 64] [--requests 200] [--loads 0.9,1.0,1.05,1.1] [--workers 4]

Batched form: `count` proofs whose sizes are drawn log-uniformly from
2^12..2^18 compressions (seeds 0..count-1) go through one server with
several workers (flock_prove_batch); the same proofs are made one after
another on one plain context. Both aggregate compressions/s are reported and
every batched proof must equal its plain proof byte for byte.

Served form: requests with sizes log-uniform in 2^10..2^20 arrive as a
Poisson process at each swept offered load (a multiple of the plain path's
compressions/s on the same mix); the server admits them by device-memory
budget and overlaps their work. Reported per rate: p50/p99 latency (submit to
proof ready) against the stated bound P99_BOUND_MS, sustained compressions/s,
the plain path's compressions/s on the same requests proven one after another
(plain_same_mix), that every served proof equals the plain proof of the same
request byte for byte (every size), and that every served proof verifies
(flock_verify_batch, with its throughput). The summary names the highest rate
whose p99 meets the bound and its sustained rate against plain_same_mix.
"""
import argparse
import json
import math
import threading
import time

import numpy as np

from . import Blake3Setup, Server, footprint_bytes, verify_batch


# The served form's latency bound: p99 of submit-to-proof time, four times
# the time a proof of the largest request size (2^20 compressions, about
# 0.1 s on the plain path) takes alone. The p99 of the mix is set by those
# largest requests, which share the GPU with the others.
P99_BOUND_MS = 400.0


def log_uniform_sizes(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return [int(math.floor(rng.uniform(lo, hi + 1))) for _ in range(n)]


class PlainProver:
    """One plain context per size (the plain path's own caches), proofs in sequence."""

    def __init__(self):
        self.setups = {}

    def prove(self, log2, seed):
        if log2 not in self.setups:
            self.setups[log2] = Blake3Setup(1 << log2)
        return self.setups[log2].prove_seed(seed)


def run_batched(count=64, workers=4, seed=20260, plain=None):
    sizes = log_uniform_sizes(count, 12, 18, seed)
    seeds = list(range(count))
    total = sum(1 << l for l in sizes)
    plain = plain or PlainProver()
    for l in sorted(set(sizes)):          # warm caches (statement digests, buffers)
        plain.prove(l, 10**6)
    t = time.perf_counter()
    ref = [plain.prove(l, s) for l, s in zip(sizes, seeds)]
    t_plain = time.perf_counter() - t
    with Server(workers=workers) as srv:
        srv.prove_batch(sorted(set(sizes)), [10**6] * len(set(sizes)))   # warm the workers
        t = time.perf_counter()
        got = srv.prove_batch(sizes, seeds)
        t_batch = time.perf_counter() - t
    same = all(a == b for a, b in zip(got, ref))
    verified = all(verify_batch(got))
    return {"proofs": count, "sizes_log2": "log-uniform 12..18", "compressions": total, "workers": workers,
            "batched_compressions_per_s": total / t_batch, "plain_sequential_compressions_per_s": total / t_plain,
            "speedup_vs_plain": t_plain / t_batch, "byte_identical_to_plain": same,
            "all_verified": verified}


def run_serving(loads=(0.9, 1.0, 1.05, 1.1), requests=200, workers=4, budget_gb=120, seed=777, plain=None,
                p99_bound_ms=P99_BOUND_MS):
    """Open-loop serving at offered loads given as multiples of the plain
    path's compressions/s on the same request mix. One mix of requests
    (sizes log-uniform 2^10..2^20, seeds) and one sequence of exponential
    gaps serve every load; a load only rescales the gaps."""
    budget = int(budget_gb * (1 << 30))
    plain = plain or PlainProver()
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(requests, 10, 20, seed)
    seeds = [int(x) for x in rng.integers(0, 2**62, requests)]
    unit_gaps = rng.exponential(1.0, requests)
    total = sum(1 << l for l in sizes)
    for l in range(10, 21):  # warm the plain path at every size (statement digests, buffers)
        plain.prove(l, 10**6)
    # the plain path on the same requests, one after another
    t = time.perf_counter()
    ref = [plain.prove(l, s) for l, s in zip(sizes, seeds)]
    t_plain = time.perf_counter() - t
    plain_cps = total / t_plain
    out = []
    for load in loads:
        rate = load * plain_cps * requests / total  # requests per second
        gaps = unit_gaps / rate
        with Server(workers=workers, hbm_budget=budget) as srv:
            srv.prove_batch(sorted(set(sizes)), [1] * len(set(sizes)))   # warm the workers
            ids, lat, proofs = [], {}, {}
            lock = threading.Lock()
            t0 = time.perf_counter()

            def collect():
                pending = set()
                while True:
                    with lock:
                        pending |= {i for i in ids if i not in lat and i not in pending}
                        finished_submitting = len(ids) == requests
                    for i in list(pending):
                        tm = srv.times(i)
                        if tm is not None:
                            lat[i] = tm[0] + tm[1]
                            proofs[i] = srv.wait(i)
                            pending.discard(i)
                    if finished_submitting and not pending and len(lat) == requests:
                        return
                    time.sleep(0.0005)

            th = threading.Thread(target=collect)
            th.start()
            nxt = t0
            for k in range(requests):
                nxt += gaps[k]
                d = nxt - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                rid = srv.submit_seed(sizes[k], seeds[k])
                with lock:
                    ids.append(rid)
            th.join()
            wall = time.perf_counter() - t0
        lats = np.array([lat[i] for i in ids])
        same = all(proofs[i] == r for i, r in zip(ids, ref))
        t = time.perf_counter()
        verified = all(verify_batch([proofs[i] for i in ids]))
        verify_s = time.perf_counter() - t
        p99 = float(np.percentile(lats, 99))
        sustained = total / wall
        out.append({"offered_over_plain": load, "rate_per_s": rate, "requests": requests,
                    "sizes_log2": "log-uniform 10..20",
                    "p50_ms": float(np.percentile(lats, 50)), "p99_ms": p99, "p99_bound_ms": p99_bound_ms,
                    "meets_p99_bound": p99 <= p99_bound_ms,
                    "sustained_compressions_per_s": sustained, "offered_compressions_per_s": total / gaps.sum(),
                    "plain_same_mix_compressions_per_s": plain_cps, "served_over_plain_same_mix": sustained / plain_cps,
                    "workers": workers, "hbm_budget_gb": budget_gb, "byte_identical_to_plain": same,
                    "all_verified": verified, "verify_proofs_per_s": requests / verify_s})
    ok = [e for e in out if e["meets_p99_bound"]]
    best = max(ok, key=lambda e: e["sustained_compressions_per_s"]) if ok else None
    summary = {"p99_bound_ms": p99_bound_ms, "plain_same_mix_compressions_per_s": plain_cps,
               "best_rate_within_bound": best["rate_per_s"] if best else None,
               "sustained_compressions_per_s": best["sustained_compressions_per_s"] if best else None,
               "sustained_over_plain_same_mix": best["served_over_plain_same_mix"] if best else None,
               "byte_identical_to_plain_all_sizes": all(e["byte_identical_to_plain"] for e in out)}
    return {"summary": summary, "rates": out}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--loads", default="0.9,1.0,1.05,1.1",
                    help="offered loads as multiples of the plain path's compressions/s on the same mix")
    ap.add_argument("--bound", type=float, default=P99_BOUND_MS, help="p99 latency bound (ms)")
    ap.add_argument("--budget-gb", type=float, default=120, help="server device-memory budget (GiB)")
    ap.add_argument("--workers", type=int, default=4)
    a = ap.parse_args(argv)
    plain = PlainProver()
    res = {"batched": run_batched(a.batch, a.workers, plain=plain),
           "serving": run_serving([float(x) for x in a.loads.split(",")], a.requests, a.workers, a.budget_gb,
                                  plain=plain, p99_bound_ms=a.bound)}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
