"""Benchmark: verified BLAKE3 compressions/s at 2^18 per proof on one GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--log2 L] [--no-forms]

Workload (the ranked configuration): one proof of 2^18 BLAKE3 compressions
per step, inputs drawn by the reference generator
(benchmark-tools/common/src/lib.rs:20-33, run on the device) from a per-step
64-bit seed. A step is the whole prover: witness, PCS commit, zerocheck,
lincheck, ring switch, Ligerito opening and serialization of the proof
bundle. The score of the reference is 2^18 / median proof time
(README.md:14-25); here every timed proof is also checked against the
deterministic re-proof of its inputs (length and bytes), and one GPU proof is
accepted by the CPU verifier in the cpu_baseline leg.

value: device-timed (CUDA events on the prover's stream) with the inputs
  already resident in HBM (flock_prove_device).
e2e:   the public C ABI with a pinned host input buffer (flock_prove): the
  28 MB input copy host->device and the proof bytes device->host are inside
  the timer. Like a worker with one pinned staging buffer, each step's own
  input is written into the same pinned buffer before its timer starts
  (rotating through one pinned 28 MB buffer per step instead made the
  copy's time vary by up to 2 ms a step on Grace hosts, while one reused
  buffer stays within 0.1 ms of the device-input proof).
Working set > 5 GB (1 GiB codeword, 0.5 GiB witness planes) >> 129 MB L2, so no
explicit L2 flush is needed between steps.
chain: the hash-chain proof of 2^18 linked compressions (flock_prove_chain),
  median of 5, and its verification (flock_verify_chain).
forms: the batched form (64 proofs of 2^12..2^18 through the proof server vs
  the same proofs in sequence) and the served form (Poisson arrivals of
  2^10..2^20 proofs, p50/p99 latency); see flock_challenge_gb300/forms.py.

--impl reference times the CPU oracle (a C++ restatement of the reference
prover path with the reference's PMULL carry-less product on Arm hosts; the
reference's Rust cannot be built here) on all host cores, on a bounded sample
of the same workload: a few full proofs of 2^18 compressions.
Under torchrun (N > 1) each rank proves its own independent batches
(replicas; proofs never shard) and rank 0 prints the line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "verified BLAKE3 compressions/s at 2^18 per proof"
PUBLISHED = 483866.0  # README.md:110-116, unmodified reference, Apple M4 Pro runner

# Figures from ncu captures of the same kernels on smaller cases (the capture
# commands and tables are kept with the other ncu summaries of the project);
# DRAM traffic and instruction counts grow in proportion to the positions.
#
# L0 commit NTT: DRAM bytes (read + write) per pass at 2^18 positions x 64
# lanes, mean of the eight L0 passes; times 4 for the bench's 2^20 positions.
NTT_TRAFFIC_PER_PASS = {20: 4 * 478.8e6}
# layers per pass of the autotuner's pass shapes (3: the deep-table pass of
# the last three layers)
NTT_MAX_LAYERS = {0: 4, 1: 6, 2: 8, 3: 3}
NTT_DEEP_SHAPE = 3
# Thread instructions per GF(2^128) product in the table passes (mean of the
# passes over layers 1..8; deeper passes spend more on their table builds), per
# butterfly in the multiply pass (its layers are the three deepest, whose
# narrow twiddles take 4 or 6 32-bit carry-less pieces) and per butterfly in
# the deep-table pass that replaces it (tables of the narrow twiddles'
# products for two of those layers), 2^18-position L0 transform.
NTT_INSTR_PER_TABLE_PRODUCT = 160
NTT_INSTR_PER_MULTIPLY_BUTTERFLY = 259
NTT_INSTR_PER_DEEP_BUTTERFLY = 148
# Zerocheck round 1 at m = 30 (2^17 outer blocks of 128 rows): warp
# instructions and DRAM bytes (read + write) of one launch, per outer block.
ZC1_WARP_INSTR_PER_OUTER = 603870960 / 2**17
ZC1_DRAM_BYTES_PER_OUTER = (419600128 + 3706624) / 2**17


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region:
    one nvidia-smi process in its own sampling loop (-lms 200), read line by
    line, rather than a process started per sample."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._p = None
        self._t = None

    def _read(self):
        for line in self._p.stdout:
            out = line.strip()
            if out:
                self.samples.append([x.strip() for x in out.split(",")])

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                        "--format=csv,noheader,nounits", "-lms", "200"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._p = None
            return self
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        if self._p is None:
            return
        self._p.terminate()
        try:
            self._p.wait(timeout=10)
        except subprocess.TimeoutExpired:
            self._p.kill()
            self._p.wait()
        self._t.join(timeout=10)

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = sorted(v for v in (num(s[0]) for s in self.samples) if v is not None)
        mx = max((v for v in (num(s[1]) for s in self.samples) if v is not None), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 2 + i and s[2 + i] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def max_over_ranks(vals, ws, device=None):
    """Each timing's maximum over the ranks (all_reduce MAX); the values unchanged on one rank."""
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def job_throughput(units_per_rank, ws, ms):
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * ws / (ms * 1e-3)


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_config(log2, ws):
    """The workload description both arms print (the same dict on each)."""
    # the prover's device working set scales with the compressions: ~7.5 GiB at 2^18
    ws_gb = 7.5 * 1.073741824 * 2.0 ** (log2 - 18)
    l2 = f"working set ~{ws_gb:.3g} GB, {'larger' if ws_gb > 0.129 else 'smaller'} than the 129 MB L2"
    return {"workload": f"one proof of 2^{log2} BLAKE3 compressions per step (m={14 + log2}, rate 1/2, "
                        "64 lanes, Fast profile, BLAKE3 Merkle + transcript, inputs from the reference "
                        "generator)",
            "parallelism": f"replicas x{ws}", "l2": l2}


def oracle_baseline(log2=18, proofs=2, gpu_proof=None, gpu_m=None):
    """CPU oracle proofs of 2^log2 compressions on all host cores (bounded
    sample: `proofs` timed proofs after the setup is cached).

    This leg is the only part of the benchmark that runs the oracle: it times
    the oracle prover and, as the checker, runs the oracle verifier on one
    proof made by the GPU arm."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    cores = os.cpu_count() or 1
    checked = None
    if gpu_proof is not None:
        ok, why = O.verify(gpu_proof, gpu_m)
        if not ok:
            raise SystemExit(f"GPU proof rejected by the CPU verifier: {why}")
        checked = f"GPU proof of m={gpu_m} ({len(gpu_proof)} bytes) accepted by the CPU verifier"
    t = time.perf_counter()
    O.warm(14 + log2)  # base matrices and statement digest, cached as the reference's setup is
    setup_s = time.perf_counter() - t
    times = []
    for i in range(proofs):
        blocks = O.compressions(log2, 1_000_000 + i)
        t = time.perf_counter()
        O.prove(blocks, log2)
        times.append(time.perf_counter() - t)
    med = statistics.median(times)
    arith = "PMULL carry-less product (the reference's aarch64 field backend)" if O.uses_pmull() else \
        "portable carry-less product"
    out = {"value": (1 << log2) / med, "unit": "compressions/s", "cores": cores, "kind": "port",
           "sample": f"{len(times)} full oracle proofs of 2^{log2} compressions (m={14 + log2}), median "
                     f"{med:.2f} s per proof ({', '.join(f'{x:.2f}' for x in times)} s), OpenMP on {cores} host "
                     f"threads, {arith}; setup (matrices + statement digest) {setup_s:.1f} s outside the timer",
           "seconds_per_proof": times}
    if checked:
        out["gpu_proof_check"] = checked
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cb = oracle_baseline(log2=args.log2, proofs=args.ref_proofs)
    med_ms = statistics.median(cb["seconds_per_proof"]) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "compressions/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": med_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": cb["value"] / PUBLISHED,
            "dtype": "u32/gf2_128", "data": "synthetic (reference input generator)",
            "config": workload_config(args.log2, ws),
            "timed_steps_note": f"each of the {len(cb['seconds_per_proof'])} timed steps is one full CPU proof "
                                f"of the workload (a bounded sample; --steps does not change it)",
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "compressions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def kernel_microbench(F, ctx_handle, peaks, torch, dev, rows_logs=(16, 18, 20), reps=3):
    """The kernel microbench shape (no protocol): rows x 256 columns of uniform
    F128, rate 1/4 (two replica layers, then the NTT), BLAKE3 Merkle over 4 KiB
    leaves. flock_commit (NTT + tree) and flock_merkle_tree are timed alone with
    CUDA events on their stream; the NTT time is their difference."""
    out = []
    s = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(s.cuda_stream)
    for rl in rows_logs:
        cols_log, rate = 8, 2
        m = 7 + cols_log + rl
        log_d = rl + rate
        z = torch.randint(-2**62, 2**62, ((1 << (rl + cols_log)) * 2,), dtype=torch.int64, device=dev).view(torch.uint8)
        cw = torch.empty((1 << (log_d + cols_log)) * 16, dtype=torch.uint8, device=dev)
        tree = torch.empty((2 * (1 << log_d) - 1) * 32, dtype=torch.uint8, device=dev)
        root = (ctypes.c_uint8 * 32)()
        lib = F.lib()

        def commit():
            F.check(lib.flock_commit(ctx_handle, F._dptr(z), m, rate, cols_log, F._dptr(cw), F._dptr(tree), root, sp),
                    "flock_commit")

        def merkle():
            F.check(lib.flock_merkle_tree(F._dptr(cw), 1 << log_d, 16 << cols_log, F._dptr(tree), sp),
                    "flock_merkle_tree")

        def timed(fn):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                fn()
                fn()
                e0.record(s)
                for _ in range(reps):
                    fn()
                e1.record(s)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        c_ms, m_ms = timed(commit), timed(merkle)
        ntt_ms = max(c_ms - m_ms, 1e-6)
        elems = (1 << (rl + cols_log))
        alg = 16 * elems * (1 + (1 << rate))  # read the message once, write the codeword once
        muls = (log_d - rate) * (1 << (log_d - 1)) * (1 << cols_log)
        leaves = 1 << log_d
        comp = leaves * ((16 << cols_log) // 64 + (16 << cols_log) // 1024 - 1) + leaves - 1
        out.append({"rows": 1 << rl, "columns": 1 << cols_log, "rate": "1/4", "leaf_bytes": 16 << cols_log,
                    "commit_ms": c_ms, "merkle_ms": m_ms, "ntt_ms": ntt_ms,
                    "ntt_gbs": alg / (ntt_ms * 1e-3) / 1e9, "ntt_frac_of_hbm": alg / (ntt_ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
                    "ntt_gf128_muls_per_s": muls / (ntt_ms * 1e-3),
                    "merkle_gbs": (16 * elems * (1 << rate)) / (m_ms * 1e-3) / 1e9,
                    "merkle_compressions_per_s": comp / (m_ms * 1e-3)})
        del z, cw, tree
        torch.cuda.empty_cache()
    return out


def ntt_l0_structure(F, dev_index, log_d):
    """(table passes, total passes, table-pass end layer, multiply-pass shape) of
    the L0 commit NTT as the library's autotuner chose them: two-layer
    byte-table passes from layer 1 to the tuned end layer, then multiply passes
    of the tuned shape (the untuned default when the shape has not run)."""
    L = F.lib()
    L.flock_ntt_tuned_variant.argtypes = [ctypes.c_int] * 4
    L.flock_ntt_tuned_table_end.argtypes = [ctypes.c_int] * 4
    variant = L.flock_ntt_tuned_variant(dev_index, log_d, 6, 1)
    max_f = NTT_MAX_LAYERS.get(variant, 6)
    tab_end = L.flock_ntt_tuned_table_end(dev_index, log_d, 6, 1)
    if tab_end < 0:  # the default depth: blocks of >= 2^9 quad-lanes
        tab_end = 1
        while tab_end + 1 < log_d and log_d - tab_end - 2 + 6 >= 9:
            tab_end += 2
    tab_passes = (tab_end - 1) // 2
    passes = tab_passes + (log_d - tab_end + max_f - 1) // max_f
    return tab_passes, passes, tab_end, variant, max_f


def rooflines(F, log2, span_ms, peaks, sms, clock_mhz, dev_index):
    """Roofline figures of the proof's main kernels from their CUDA-event times
    inside the timed proofs (mean over the timed steps, on the prover's stream).

    Algorithmic bytes follow the hot-path measurement rules: the NTT reads the
    message once and writes the codeword once (16 B x rows x 64 lanes x (1 + 2));
    zerocheck round 1 reads a, b and z once (3 x 2^m / 8 bytes); the witness
    writes z, a, b and the stripe (4 x 2,048 B) and reads 112 B per compression.
    `traffic` is the ncu DRAM traffic per launch (set) scaled to this size;
    `integer_frac` is thread instructions (ncu counts) over the same time
    against the SM issue peak, SMs x 4 x 32 lanes x SM clock."""
    m = 14 + log2
    log_d = m - 7 - 6 + 1
    hbm = peaks["hbm_gbs"]
    clock = clock_mhz or peaks.get("sm_max_mhz", 2070.0)
    issue_peak = sms * 4 * 32 * clock * 1e6
    out = {}
    # L0 commit NTT
    ms = span_ms["l0_ntt"]
    tab_passes, passes, tab_end, variant, max_f = ntt_l0_structure(F, dev_index, log_d)
    msg = (1 << (log_d - 1)) * 64 * 16
    alg = msg + 2 * msg  # message read once + codeword written once
    traffic = passes * NTT_TRAFFIC_PER_PASS[log_d] if log_d in NTT_TRAFFIC_PER_PASS else None

    def products(l):  # butterflies of layer l with a product (block 0 skips it)
        return ((1 << (log_d - 1)) - (1 << (log_d - l - 1))) * 64
    deep = variant == NTT_DEEP_SHAPE
    ins = (sum(products(l) for l in range(1, tab_end)) * NTT_INSTR_PER_TABLE_PRODUCT
           + sum(products(l) for l in range(tab_end, log_d))
           * (NTT_INSTR_PER_DEEP_BUTTERFLY if deep else NTT_INSTR_PER_MULTIPLY_BUTTERFLY))
    last = ("the deep-table pass of the last 3 layers" if deep
            else f"{passes - tab_passes} multiply pass(es) of <= {max_f} layers")
    muls = sum(products(l) for l in range(1, log_d))
    out["l0_ntt"] = {
        "kernel": f"L0 commit NTT, layers 1..{log_d - 1} of 2^{log_d} positions x 64 lanes ({tab_passes} two-layer "
                  f"table passes, then {last})",
        "bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
        "frac": alg / (ms * 1e-3) / 1e9 / hbm, "traffic": traffic,
        "algorithmic_bytes": alg, "traffic_over_algorithmic": (traffic / alg) if traffic else None,
        "integer_frac": ins / (ms * 1e-3) / issue_peak, "integer_achieved_tips": ins / (ms * 1e-3) / 1e12,
        "integer_peak_tips": issue_peak / 1e12, "ms_per_launch_set": ms, "passes": passes,
        "gf128_products_per_s": muls / (ms * 1e-3), "pass_shape": variant}
    # zerocheck round 1
    ms = span_ms["zerocheck_round1"]
    n_outer = (1 << m) // 64 // 128
    alg = 3 * (1 << m) // 8
    ins = ZC1_WARP_INSTR_PER_OUTER * 32 * n_outer
    traffic = ZC1_DRAM_BYTES_PER_OUTER * n_outer
    out["zerocheck_round1"] = {
        "kernel": f"zerocheck univariate-skip round 1 over 2^{m - 6} rows of a, b, z",
        "bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
        "frac": alg / (ms * 1e-3) / 1e9 / hbm, "traffic": traffic, "algorithmic_bytes": alg,
        "traffic_over_algorithmic": traffic / alg, "integer_frac": ins / (ms * 1e-3) / issue_peak,
        "integer_achieved_tips": ins / (ms * 1e-3) / 1e12, "ms_per_launch": ms}
    # witness
    ms = span_ms["witness"]
    alg = (1 << log2) * (112 + 4 * 2048)
    out["witness"] = {"kernel": f"witness z, a, b and lincheck stripe of 2^{log2} compressions", "bound": "hbm",
                      "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                      "frac": alg / (ms * 1e-3) / 1e9 / hbm, "algorithmic_bytes": alg, "ms_per_launch": ms}
    return out


def run_chain(F, setup, log2, reps=5):
    """Hash-chain proof (flock_prove_chain, host inputs in, bundle bytes out) of
    2^log2 linked compressions built as the flock_chain CLI builds them."""
    import statistics
    blocks = F.chain_inputs(1 << log2, 42)
    first = setup.prove_chain(blocks)  # warm-up: the chain tables are allocated here
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        b = setup.prove_chain(blocks)
        ts.append((time.perf_counter() - t0) * 1e3)
        if b != first:
            raise SystemExit("chain proof not deterministic")
    t0 = time.perf_counter()
    ok = F.verify_chain(first, ctx=setup.ctx)
    v_ms = (time.perf_counter() - t0) * 1e3
    if not ok:
        raise SystemExit("a chain proof was rejected by flock_verify_chain")
    ms = statistics.median(ts)
    return {"workload": f"BLAKE3 chain of 2^{log2} compressions (flock_chain CLI inputs, domain flock_chain-cli)",
            "impl": "flock_prove_chain, host inputs -> bundle bytes", "ms_per_proof": ms,
            "compressions_per_s": (1 << log2) / (ms * 1e-3), "proof_bytes": len(first),
            "verify_ms": v_ms, "accepted": ok, "reps": reps}


def run_gpu(args):
    import statistics

    import numpy as np
    import torch
    import flock_challenge_gb300 as F

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    log2 = args.log2
    n = 1 << log2
    setup = F.Blake3Setup(n, device=local)
    stream = torch.cuda.ExternalStream(setup.stream_handle(), device=dev)
    nseeds = max(args.steps, 1)
    # per-step inputs: the reference generator (benchmark-tools/common/src/lib.rs:20-33),
    # run on the device; host copies feed the end-to-end leg through one pinned buffer
    d_seeded = [F.generate_inputs(log2, 1000 * rank + i, device=dev) for i in range(nseeds)]
    host = [d.cpu() for d in d_seeded]
    pin_in = torch.empty_like(host[0]).pin_memory()
    L = F._proto_lib()
    obuf = np.zeros(1 << 20, np.uint8)

    def prove_host(h):
        """flock_prove with a pinned host buffer: the input copy is inside the call."""
        ln = ctypes.c_size_t()
        F.check(L.flock_prove(setup.ctx.handle, ctypes.c_void_p(h.data_ptr()), n,
                              obuf.ctypes.data_as(ctypes.c_void_p), obuf.size, ctypes.byref(ln)), "flock_prove")
        return ln.value

    # warm-up (untimed, like the reference worker's fixed-seed proof), then the
    # proof of every step's input, against which the timed proofs are checked
    for i in range(args.warmup):
        setup.prove_device(d_seeded[i % nseeds])
    expected = [setup.prove_device(d) for d in d_seeded]
    # the host-buffer and seed paths warm up too (their staging buffers)
    for h in host[:3]:
        pin_in.copy_(h)
        prove_host(pin_in)
    setup.prove_seed(999_999)
    setup.set_kernel_timing(True)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    spans = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        launches0 = F.kernel_launches()
        ev[0].record(stream)
        for i in range(args.steps):
            p = setup.prove_device(d_seeded[i])
            ev[i + 1].record(stream)
            spans.append(setup.kernel_times())
            assert p == expected[i]  # deterministic, full-length proof bytes of this step's input
        torch.cuda.synchronize()
        launches = F.kernel_launches() - launches0
        step_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
        dev_ms = ev[0].elapsed_time(ev[-1]) / args.steps
        phases = setup.phase_times()
        setup.set_kernel_timing(False)
        # End to end through the public C ABI: the step's input is written into
        # the pinned input buffer, then the timer covers flock_prove (input copy
        # in, proof, proof bytes out); the bytes are checked after the timer.
        torch.cuda.synchronize()
        sizes, e2e_steps, e2e_same = [], [], True
        for i in range(args.steps):
            pin_in.copy_(host[i])
            ts = time.perf_counter()
            sizes.append(prove_host(pin_in))
            e2e_steps.append((time.perf_counter() - ts) * 1e3)
            e2e_same = e2e_same and obuf[:sizes[-1]].tobytes() == expected[i]
        torch.cuda.synchronize()
        e2e_ms = statistics.fmean(e2e_steps)
        # Seed to proof bytes (the reference worker's timed path): inputs generated on the device.
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            setup.prove_seed(1000 * rank + i)
        torch.cuda.synchronize()
        seed_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if sizes != [len(e) for e in expected] or not e2e_same:
        raise SystemExit("an end-to-end proof differs from the device-input proof of the same seed")
    # every timed proof checked by the device-accelerated verifier (outside the timer)
    t0 = time.perf_counter()
    verified = all(F.verify(p, ctx=setup.ctx) for p in expected)
    verify_ms = (time.perf_counter() - t0) * 1e3 / len(expected)
    if not verified:
        raise SystemExit("a timed proof was rejected by flock_verify")
    peaks, src = load_peaks()
    span_mean = {k: statistics.fmean(s[k] for s in spans) for k in F.KERNEL_SPANS}
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roofs = rooflines(F, log2, span_mean, peaks, sms, clk.summary().get("sm_mhz"), dev.index or 0)
    dev_ms, e2e_ms, seed_ms = max_over_ranks([dev_ms, e2e_ms, seed_ms], ws, device=dev)
    if rank == 0:
        total = n * ws
        med_ms = statistics.median(step_ms)
        roof = dict(roofs["l0_ntt"])
        roof["peak_source"] = f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else src
        line = {
            "metric": METRIC, "value": job_throughput(n, ws, dev_ms), "unit": "compressions/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": (total / (dev_ms * 1e-3)) / PUBLISHED,
            "dtype": "u32/gf2_128", "data": "synthetic (reference input generator, one seed per step)",
            "config": workload_config(log2, ws),
            "median": {"ms_per_step": med_ms, "value": job_throughput(n, ws, med_ms),
                       "note": "the reference's score is 2^18 / median trial time"},
            "step_ms": [round(x, 3) for x in step_ms],
            "proof": {"bytes_first_step": len(expected[0]),
                      "verified": "every timed proof byte-equal to the untimed proof of the same input and "
                                  "accepted by flock_verify; one also by the CPU verifier (cpu_baseline)",
                      "phase_ms_last_proof": {k: round(v, 3) for k, v in phases.items()},
                      "kernel_ms_mean": {k: round(v, 4) for k, v in span_mean.items()}},
            "e2e": {"value": job_throughput(n, ws, e2e_ms), "unit": "compressions/s", "h2d_bytes_per_step": n * 112,
                    "d2h_bytes_per_step": len(expected[0]), "step_ms": [round(x, 3) for x in e2e_steps],
                    "median_ms": statistics.median(e2e_steps),
                    "input": "the step's own input in one pinned host buffer (written before the timer); "
                             "proof bytes equal to the device-input proof of the same seed"},
            "e2e_seed_to_proof": {"value": job_throughput(n, ws, seed_ms), "unit": "compressions/s",
                                  "h2d_bytes_per_step": 8, "d2h_bytes_per_step": len(expected[0]),
                                  "note": "seed in, inputs generated on the device, proof bytes out"},
            "verify": {"impl": "flock_verify (host transcript + device kernels)", "ms_per_proof": verify_ms,
                       "accepted": verified, "proofs": len(expected)},
            "gpu_launches": int(launches),
            "roofline": roof,
            "roofline_kernels": roofs,
            "clocks": clk.summary(),
        }
        if ws == 1:
            line["chain"] = run_chain(F, setup, log2)
            line["kernel_microbench"] = kernel_microbench(F, setup.ctx.handle, peaks, torch, dev,
                                                          rows_logs=tuple(args.micro_rows))
        line["cpu_baseline"] = oracle_baseline(log2=log2, proofs=args.cpu_proofs, gpu_proof=expected[0],
                                               gpu_m=14 + log2)
        if args.forms and ws == 1:
            from flock_challenge_gb300 import forms
            plain = forms.PlainProver()
            line["forms"] = {"batched": forms.run_batched(64, 4, plain=plain),
                             "serving": forms.run_serving((0.9, 1.0, 1.05, 1.1), 200, 4, plain=plain)}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log2", type=int, default=18)
    ap.add_argument("--forms", dest="forms", action="store_true", default=True,
                    help="also measure the batched and served forms (default)")
    ap.add_argument("--no-forms", dest="forms", action="store_false")
    ap.add_argument("--cpu-proofs", type=int, default=2, help="timed CPU oracle proofs in the cpu_baseline leg")
    ap.add_argument("--ref-proofs", type=int, default=3, help="timed CPU oracle proofs of the reference arm")
    ap.add_argument("--micro-rows", type=int, nargs="*", default=[16, 18, 20, 22],
                    help="log2 rows of the kernel microbench (256 columns, rate 1/4)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
