"""GB300-native (sm_103a) prover hot path for batched BLAKE3 compressions.

Host-side mirror of the reference's prover entry points
(crates/flock-prover/src/r1cs_hashes/blake3.rs `Blake3Setup`, and
crates/flock-core/src/pcs/commit.rs `commit`) over the C ABI of
include/flock_gpu.h, implemented by libflock_gpu.so (CUDA, built in-tree).

There is no CPU fallback: importing the native library fails loudly when it
is missing or cannot be loaded.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None

COMPRESSION_DTYPE = np.dtype([("cv", "<u4", 8), ("m", "<u4", 16), ("counter", "<u8"),
                              ("block_len", "<u4"), ("flags", "<u4")])
assert COMPRESSION_DTYPE.itemsize == 112

FLOCK_OK = 0
FLOCK_PENDING = 1
_ERRORS = {-1: "shape", -2: "cuda", -3: "out of memory", -4: "argument", -5: "capacity",
           -6: "timeout", -7: "verify", -8: "limit"}


class FlockError(RuntimeError):
    pass


def check(rc, what="flock call"):
    if rc != FLOCK_OK:
        raise FlockError(f"{what} failed: {_ERRORS.get(rc, rc)} ({rc})")


def lib_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Loads libflock_gpu.so (building it first when sources are newer)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise FlockError(f"native library missing: {_build.LIB}")
    L = ctypes.CDLL(_build.LIB)
    P, sz, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    L.flock_version.restype = ctypes.c_char_p
    L.flock_create.argtypes = [i32, sz, ctypes.POINTER(P)]
    L.flock_destroy.argtypes = [P]
    L.flock_witness.argtypes = [P, sz, i32, P, P, P, P, P]
    L.flock_ntt.argtypes = [P, P, i32, i32, i32, P]
    L.flock_merkle_tree.argtypes = [P, sz, sz, P, P]
    L.flock_commit.argtypes = [P, P, i32, i32, i32, P, P, P, P]
    _LIB = L
    return L


class Context:
    """Device context (flock_create / flock_destroy)."""

    def __init__(self, device=0, hbm_budget=0):
        self._h = ctypes.c_void_p()
        check(lib().flock_create(device, hbm_budget, ctypes.byref(self._h)), "flock_create")
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().flock_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream_ptr(stream):
    return ctypes.c_void_p(stream.cuda_stream) if stream is not None else None


def generate_witness(d_blocks, n, n_blocks_log, want_ab=True, want_stripe=True, stream=None):
    """Witness (z, a, b, stripe) on the device for n compressions in 2^n_blocks_log slots.

    d_blocks: uint8 CUDA tensor of n * 112 bytes (flock_compression records).
    Returns torch uint8 CUDA tensors (a/b/stripe None when not requested).
    """
    import torch
    m = 14 + n_blocks_log
    nbytes = (1 << m) // 8
    dev = d_blocks.device
    z = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    a = torch.empty(nbytes, dtype=torch.uint8, device=dev) if want_ab else None
    b = torch.empty(nbytes, dtype=torch.uint8, device=dev) if want_ab else None
    s = torch.empty(nbytes, dtype=torch.uint8, device=dev) if want_stripe else None
    check(lib().flock_witness(_dptr(d_blocks), n, n_blocks_log, _dptr(z), _dptr(a), _dptr(b), _dptr(s),
                              _stream_ptr(stream)), "flock_witness")
    return z, a, b, s


def commit(ctx, d_z, m, log_inv_rate=1, log_batch_size=6, stream=None):
    """PCS commit on the device: returns (root bytes, codeword tensor, tree tensor)."""
    import torch
    log_d = m - 7 - log_batch_size + log_inv_rate
    cw = torch.empty((1 << (log_d + log_batch_size)) * 16, dtype=torch.uint8, device=d_z.device)
    tree = torch.empty((2 * (1 << log_d) - 1) * 32, dtype=torch.uint8, device=d_z.device)
    root = (ctypes.c_uint8 * 32)()
    check(lib().flock_commit(ctx.handle, _dptr(d_z), m, log_inv_rate, log_batch_size, _dptr(cw), _dptr(tree),
                             root, _stream_ptr(stream)), "flock_commit")
    return bytes(root), cw, tree


def ntt(ctx, d_data, log_d, log_num_ntts, start_layer=0, stream=None):
    check(lib().flock_ntt(ctx.handle, _dptr(d_data), log_d, log_num_ntts, start_layer, _stream_ptr(stream)),
          "flock_ntt")


def merkle_tree(d_data, n_leaves, leaf_bytes, stream=None):
    import torch
    tree = torch.empty((2 * n_leaves - 1) * 32, dtype=torch.uint8, device=d_data.device)
    check(lib().flock_merkle_tree(_dptr(d_data), n_leaves, leaf_bytes, _dptr(tree), _stream_ptr(stream)),
          "flock_merkle_tree")
    return tree


def _proto_lib():
    L = lib()
    if not getattr(L, "_proto_ready", False):
        P = ctypes.c_void_p
        L.flock_setup.argtypes = [P, ctypes.c_size_t]
        L.flock_prove.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.flock_last_phase_times.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.flock_last_host_waits.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double),
                                            ctypes.c_int]
        L.flock_kernel_timing.argtypes = [P, ctypes.c_int]
        L.flock_set_wait_limit.argtypes = [P, ctypes.c_double]
        L.flock_last_kernel_times.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.flock_prove_seed.argtypes = [P, ctypes.c_uint32, ctypes.c_uint64, P, ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_size_t)]
        L.flock_prove_device.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.flock_generate_inputs.argtypes = [ctypes.c_uint32, ctypes.c_uint64, P, P]
        L.flock_kernel_launches.restype = ctypes.c_uint64
        L.flock_stream.argtypes = [P]
        L.flock_stream.restype = P
        u64p, szp = ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_size_t)
        L.flock_footprint_bytes.argtypes = [ctypes.c_uint32]
        L.flock_footprint_bytes.restype = ctypes.c_size_t
        L.flock_server_create.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(P)]
        L.flock_server_destroy.argtypes = [P]
        L.flock_server_submit_seed.argtypes = [P, ctypes.c_uint32, ctypes.c_uint64, u64p]
        L.flock_server_submit.argtypes = [P, P, ctypes.c_size_t, u64p]
        L.flock_server_poll.argtypes = [P, ctypes.c_uint64, P, ctypes.c_size_t, szp]
        L.flock_server_wait.argtypes = [P, ctypes.c_uint64, P, ctypes.c_size_t, szp]
        L.flock_server_request_times.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.POINTER(ctypes.c_double)]
        L.flock_server_reserved_bytes.argtypes = [P]
        L.flock_server_reserved_bytes.restype = ctypes.c_size_t
        L.flock_prove_batch.argtypes = [P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32), u64p, P,
                                        ctypes.c_size_t, szp]
        L.flock_verify.argtypes = [P, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int)]
        L.flock_verify_batch.argtypes = [P, ctypes.c_size_t, ctypes.POINTER(P), szp, ctypes.POINTER(ctypes.c_int)]
        L.flock_prove_chain.argtypes = [P, P, ctypes.c_size_t, ctypes.c_char_p, P, ctypes.c_size_t, szp]
        L.flock_verify_chain.argtypes = [P, P, ctypes.c_size_t, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.flock_chain_inputs.argtypes = [ctypes.c_size_t, ctypes.c_uint64, P, P]
        L.flock_transcript_create.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(P)]
        L.flock_transcript_fork.argtypes = [P, ctypes.POINTER(P)]
        L.flock_transcript_destroy.argtypes = [P]
        L.flock_transcript_observe_label.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
        L.flock_transcript_observe_f128.argtypes = [P, u64p]
        L.flock_transcript_observe_f128_slice.argtypes = [P, u64p, ctypes.c_size_t]
        L.flock_transcript_observe_bytes.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
        L.flock_transcript_sample_f128.argtypes = [P, u64p]
        L.flock_transcript_sample_f128_vec.argtypes = [P, ctypes.c_size_t, u64p]
        L.flock_prove_challenger.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int, P, P, ctypes.c_size_t, szp, P,
                                             ctypes.POINTER(R1csClaim)]
        L.flock_verify_challenger.argtypes = [P, P, ctypes.c_size_t, P, ctypes.POINTER(ctypes.c_int)]
        L._proto_ready = True
    return L


CLAIM_MAX_OUTER = 24  # FLOCK_CLAIM_MAX_OUTER


class ZClaim(ctypes.Structure):
    """flock_zclaim: z_hat(point) = value with point (z_skip, x_inner_rest, x_outer)
    (ZClaim / QuirkyPoint, crates/flock-core/src/proof.rs:26-29, lincheck.rs:418-426)."""
    _fields_ = [("z_skip", ctypes.c_uint64 * 2), ("x_inner_rest", (ctypes.c_uint64 * 2) * 8),
                ("x_outer", (ctypes.c_uint64 * 2) * CLAIM_MAX_OUTER), ("n_outer", ctypes.c_uint32),
                ("value", ctypes.c_uint64 * 2)]

    def as_dict(self):
        f = lambda a: (int(a[0]), int(a[1]))  # noqa: E731
        return {"z_skip": f(self.z_skip), "x_inner_rest": [f(x) for x in self.x_inner_rest],
                "x_outer": [f(self.x_outer[i]) for i in range(self.n_outer)], "value": f(self.value)}


class R1csClaim(ctypes.Structure):
    """flock_r1cs_claim: R1csClaim { ab, c } (crates/flock-core/src/proof.rs:36-45)."""
    _fields_ = [("ab", ZClaim), ("c", ZClaim)]


class FsChallenger:
    """Caller-owned Fiat-Shamir transcript (flock_transcript_*): the reference's
    FsChallenger::with_hash(domain, HashKind::Blake3)
    (crates/flock-core/src/challenger.rs:183-438). F128 values are (lo, hi) pairs."""

    def __init__(self, domain=b"flock-bench-v0", _handle=None):
        self._h = ctypes.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            d = _domain_bytes(domain)
            check(_proto_lib().flock_transcript_create(d, len(d), ctypes.byref(self._h)), "flock_transcript_create")

    @property
    def handle(self):
        return self._h

    def fork(self):
        h = ctypes.c_void_p()
        check(_proto_lib().flock_transcript_fork(self._h, ctypes.byref(h)), "flock_transcript_fork")
        return FsChallenger(_handle=h)

    def observe_label(self, label):
        b = _domain_bytes(label)
        check(_proto_lib().flock_transcript_observe_label(self._h, b, len(b)), "observe_label")

    def observe_f128(self, v):
        a = (ctypes.c_uint64 * 2)(*v)
        check(_proto_lib().flock_transcript_observe_f128(self._h, a), "observe_f128")

    def observe_f128_slice(self, vs):
        a = (ctypes.c_uint64 * (2 * max(len(vs), 1)))(*[w for v in vs for w in v])
        check(_proto_lib().flock_transcript_observe_f128_slice(self._h, a, len(vs)), "observe_f128_slice")

    def observe_bytes(self, b):
        b = bytes(b)
        check(_proto_lib().flock_transcript_observe_bytes(self._h, b, len(b)), "observe_bytes")

    def sample_f128(self):
        a = (ctypes.c_uint64 * 2)()
        check(_proto_lib().flock_transcript_sample_f128(self._h, a), "sample_f128")
        return int(a[0]), int(a[1])

    def sample_f128_vec(self, n):
        a = (ctypes.c_uint64 * (2 * max(n, 1)))()
        check(_proto_lib().flock_transcript_sample_f128_vec(self._h, n, a), "sample_f128_vec")
        return [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]

    def close(self):
        if self._h:
            _proto_lib().flock_transcript_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


KERNEL_SPANS = ["witness", "l0_ntt", "l0_merkle", "zerocheck_round1"]

PHASES = ["setup", "commit", "zerocheck_round1", "zerocheck_rounds", "lincheck", "ring_switch", "ligerito",
          "serialize"]


class Blake3Setup:
    """Prover for batched BLAKE3 compressions on one GPU.

    Mirrors crates/flock-prover/src/r1cs_hashes/blake3.rs `Blake3Setup`:
    ``Blake3Setup(n_blocks)`` then ``prove_fast(blocks)`` returning the
    serialized proof bundle (R1csProofBundleLigerito::to_bytes). Blocks are a
    numpy array of COMPRESSION_DTYPE records (cv, m, counter, block_len, flags).
    """

    def __init__(self, n_blocks, device=0):
        if n_blocks < 1:
            raise ValueError("n_blocks must be >= 1")
        self.n_blocks = n_blocks
        n = max(n_blocks, 8)
        self.n_blocks_log = (n - 1).bit_length()
        self.m = 14 + self.n_blocks_log
        self.ctx = Context(device)
        check(_proto_lib().flock_setup(self.ctx.handle, n_blocks), "flock_setup")
        self._buf = np.zeros(1 << 20, np.uint8)

    def prove_fast(self, blocks, challenger=None):
        """Proof bundle bytes of `blocks` under a fresh "flock-bench-v0" transcript;
        with `challenger` (an FsChallenger), the proof continues that transcript
        and advances it, and the call returns (bundle bytes, commitment root,
        R1csClaim as a dict), as the reference's prove_fast returns (proof,
        commitment, claim) (blake3.rs:3405-3409)."""
        blocks = np.ascontiguousarray(blocks, dtype=COMPRESSION_DTYPE)
        if len(blocks) != self.n_blocks:
            raise ValueError(f"expected {self.n_blocks} blocks, got {len(blocks)}")
        L = _proto_lib()
        if challenger is not None:
            root = (ctypes.c_uint8 * 32)()
            claim = R1csClaim()
            proof = self._call(L.flock_prove_challenger, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks), 0,
                               challenger.handle, _tail=(root, ctypes.byref(claim)))
            return proof, bytes(root), {"ab": claim.ab.as_dict(), "c": claim.c.as_dict()}
        ln = ctypes.c_size_t()
        rc = L.flock_prove(self.ctx.handle, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks),
                           self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size, ctypes.byref(ln))
        if rc == -5:
            self._buf = np.zeros(ln.value, np.uint8)
            rc = L.flock_prove(self.ctx.handle, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks),
                               self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size, ctypes.byref(ln))
        check(rc, "flock_prove")
        return self._buf[:ln.value].tobytes()

    def _call(self, fn, *args, _tail=()):
        ln = ctypes.c_size_t()
        rc = fn(self.ctx.handle, *args, self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size, ctypes.byref(ln),
                *_tail)
        if rc == -5:
            self._buf = np.zeros(ln.value, np.uint8)
            rc = fn(self.ctx.handle, *args, self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size,
                    ctypes.byref(ln), *_tail)
        check(rc, fn.__name__)
        return self._buf[:ln.value].tobytes()

    def prove_seed(self, seed):
        """Seed -> proof bytes: inputs generated on the device from `seed` with the
        reference generator (benchmark-tools/common/src/lib.rs:20-33), then proven."""
        if self.n_blocks != 1 << self.n_blocks_log:
            raise ValueError("prove_seed needs a power-of-two n_blocks")
        return self._call(_proto_lib().flock_prove_seed, self.n_blocks_log, seed)

    def prove_device(self, d_blocks):
        """Proof of n_blocks records already in device memory (uint8 CUDA tensor)."""
        return self._call(_proto_lib().flock_prove_device, ctypes.c_void_p(d_blocks.data_ptr()), self.n_blocks)

    def verify(self, proof):
        """True when `proof` (bundle bytes) verifies (flock_verify, on this context's GPU)."""
        return verify(proof, ctx=self.ctx)

    def prove_chain(self, blocks, domain=None):
        """Hash-chain proof of n_blocks = 2^k compressions whose cvs link
        (Blake3Setup::prove_chain, crates/flock-prover/src/r1cs_hashes/blake3.rs:3785-3805):
        the ChainProofBundleLigerito bytes, endpoints taken from the blocks."""
        blocks = np.ascontiguousarray(blocks, dtype=COMPRESSION_DTYPE)
        if len(blocks) != self.n_blocks or self.n_blocks != 1 << self.n_blocks_log:
            raise ValueError("prove_chain needs exactly n_blocks = 2^k blocks")
        return self._call(_proto_lib().flock_prove_chain, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks),
                          _domain_bytes(domain))

    def verify_chain(self, bundle, domain=None):
        """True when the chain bundle verifies (flock_verify_chain)."""
        return verify_chain(bundle, domain, ctx=self.ctx)

    def stream_handle(self):
        """cudaStream_t the prover launches on (for event timing)."""
        return _proto_lib().flock_stream(self.ctx.handle)

    def set_wait_limit(self, ms):
        """Bounds each host wait of this prover's later calls by `ms` milliseconds
        (0: no bound); a call whose wait passes it raises FlockError (timeout)
        and the next call first waits for its queued work (flock_set_wait_limit)."""
        check(_proto_lib().flock_set_wait_limit(self.ctx.handle, float(ms)), "flock_set_wait_limit")

    def set_kernel_timing(self, on=True):
        """CUDA-event timing of the main kernels of each proof (flock_kernel_timing)."""
        check(_proto_lib().flock_kernel_timing(self.ctx.handle, int(bool(on))), "flock_kernel_timing")

    def kernel_times(self):
        """Device ms of the last proof's main kernels (flock_last_kernel_times)."""
        arr = (ctypes.c_double * len(KERNEL_SPANS))()
        check(_proto_lib().flock_last_kernel_times(self.ctx.handle, arr, len(KERNEL_SPANS)), "flock_last_kernel_times")
        return dict(zip(KERNEL_SPANS, list(arr)))

    def phase_times(self):
        arr = (ctypes.c_double * 8)()
        check(_proto_lib().flock_last_phase_times(self.ctx.handle, arr, 8), "flock_last_phase_times")
        return dict(zip(PHASES, list(arr)))

    def host_waits(self):
        """Per phase of the last proof: (number of host waits for the stream, ms blocked in them)."""
        n = (ctypes.c_uint64 * 8)()
        ms = (ctypes.c_double * 8)()
        check(_proto_lib().flock_last_host_waits(self.ctx.handle, n, ms, 8), "flock_last_host_waits")
        return {k: (int(a), float(b)) for k, a, b in zip(PHASES, n, ms)}


def kernel_launches():
    """Number of kernels this library has launched in the process."""
    return int(_proto_lib().flock_kernel_launches())


def generate_inputs(log2_size, seed, device="cuda"):
    """The reference's 2^log2_size benchmark compressions for `seed`, generated on the device."""
    import torch
    out = torch.empty((1 << log2_size) * 112, dtype=torch.uint8, device=device)
    check(_proto_lib().flock_generate_inputs(log2_size, seed, _dptr(out), None), "flock_generate_inputs")
    return out


def footprint_bytes(log2_size):
    """Device bytes one prover holds for a proof of 2^log2_size compressions."""
    return int(_proto_lib().flock_footprint_bytes(log2_size))


class Server:
    """Proof server with continuous batching (flock_server_*).

    ``Server(device, hbm_budget, workers)``; ``submit_seed(log2, seed)`` or
    ``submit(blocks)`` return a request id; ``wait(id)`` / ``poll(id)`` return
    the proof bytes (poll returns None while the request runs). Requests are
    admitted while the workers' device memory fits ``hbm_budget`` (0 = no
    limit) and run concurrently on the workers' streams.
    """

    def __init__(self, device=0, hbm_budget=0, workers=2):
        self._h = ctypes.c_void_p()
        check(_proto_lib().flock_server_create(device, hbm_budget, workers, ctypes.byref(self._h)),
              "flock_server_create")
        self._buf = np.zeros(1 << 20, np.uint8)

    def close(self):
        if self._h:
            _proto_lib().flock_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit_seed(self, log2_size, seed):
        rid = ctypes.c_uint64()
        check(_proto_lib().flock_server_submit_seed(self._h, log2_size, seed, ctypes.byref(rid)),
              "flock_server_submit_seed")
        return rid.value

    def submit(self, blocks):
        blocks = np.ascontiguousarray(blocks, dtype=COMPRESSION_DTYPE)
        rid = ctypes.c_uint64()
        check(_proto_lib().flock_server_submit(self._h, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks),
                                               ctypes.byref(rid)), "flock_server_submit")
        return rid.value

    def _collect(self, fn, rid):
        ln = ctypes.c_size_t()
        rc = fn(self._h, rid, self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size, ctypes.byref(ln))
        if rc == -5:
            self._buf = np.zeros(ln.value, np.uint8)
            rc = fn(self._h, rid, self._buf.ctypes.data_as(ctypes.c_void_p), self._buf.size, ctypes.byref(ln))
        if rc == FLOCK_PENDING:
            return None
        check(rc, fn.__name__)
        return self._buf[:ln.value].tobytes()

    def poll(self, rid):
        return self._collect(_proto_lib().flock_server_poll, rid)

    def wait(self, rid):
        return self._collect(_proto_lib().flock_server_wait, rid)

    def times(self, rid):
        """(queue_ms, run_ms) of a finished request, before it is collected."""
        q, r = ctypes.c_double(), ctypes.c_double()
        rc = _proto_lib().flock_server_request_times(self._h, rid, ctypes.byref(q), ctypes.byref(r))
        if rc == FLOCK_PENDING:
            return None
        check(rc, "flock_server_request_times")
        return q.value, r.value

    def reserved_bytes(self):
        return int(_proto_lib().flock_server_reserved_bytes(self._h))

    def prove_batch(self, log2_sizes, seeds):
        """Batched form: one proof per (log2_size, seed), as flock_prove_seed would make it."""
        n = len(log2_sizes)
        sizes = (ctypes.c_uint32 * n)(*log2_sizes)
        sds = (ctypes.c_uint64 * n)(*seeds)
        lens = (ctypes.c_size_t * n)()
        cap = n * 600000
        out = np.zeros(cap, np.uint8)
        check(_proto_lib().flock_prove_batch(self._h, n, sizes, sds, out.ctypes.data_as(ctypes.c_void_p), cap, lens),
              "flock_prove_batch")
        proofs, off = [], 0
        for i in range(n):
            proofs.append(out[off:off + lens[i]].tobytes())
            off += lens[i]
        return proofs


_VERIFY_CTX = {}


def verify(proof, ctx=None, device=0, challenger=None):
    """flock_verify: True when the serialized proof bundle verifies.

    Mirrors verifier::verify_ligerito on R1csProofBundleLigerito::from_bytes
    (crates/flock-core/src/verifier.rs, crates/flock-prover/src/proof_io.rs).
    With `challenger` (an FsChallenger) the replay continues that transcript
    (flock_verify_challenger), which advances only on acceptance."""
    if ctx is None:
        ctx = _VERIFY_CTX.get(device)
        if ctx is None:
            ctx = _VERIFY_CTX[device] = Context(device)
    buf = np.frombuffer(bytes(proof), np.uint8)
    ok = ctypes.c_int()
    if challenger is not None:
        check(_proto_lib().flock_verify_challenger(ctx.handle, buf.ctypes.data_as(ctypes.c_void_p), buf.size,
                                                   challenger.handle, ctypes.byref(ok)), "flock_verify_challenger")
    else:
        check(_proto_lib().flock_verify(ctx.handle, buf.ctypes.data_as(ctypes.c_void_p), buf.size,
                                        ctypes.byref(ok)), "flock_verify")
    return bool(ok.value)


def verify_batch(proofs, ctx=None, device=0):
    """flock_verify_batch over a list of proof bundles: a list of booleans."""
    if ctx is None:
        ctx = _VERIFY_CTX.get(device)
        if ctx is None:
            ctx = _VERIFY_CTX[device] = Context(device)
    bufs = [np.frombuffer(bytes(p), np.uint8) for p in proofs]
    n = len(bufs)
    ptrs = (ctypes.c_void_p * n)(*[b.ctypes.data for b in bufs])
    lens = (ctypes.c_size_t * n)(*[b.size for b in bufs])
    acc = (ctypes.c_int * n)()
    check(_proto_lib().flock_verify_batch(ctx.handle, n, ptrs, lens, acc), "flock_verify_batch")
    return [bool(a) for a in acc]


def _domain_bytes(domain):
    return domain.encode() if isinstance(domain, str) else domain


def verify_chain(bundle, domain=None, ctx=None, device=0):
    """flock_verify_chain: True when the chain bundle verifies under `domain`
    (None = "flock_chain-cli"); Blake3Setup::verify_chain on
    ChainProofBundleLigerito::from_bytes (blake3.rs:3807-3830, proof_io.rs:494-497)."""
    if ctx is None:
        ctx = _VERIFY_CTX.get(device)
        if ctx is None:
            ctx = _VERIFY_CTX[device] = Context(device)
    buf = np.frombuffer(bytes(bundle), np.uint8)
    ok = ctypes.c_int()
    check(_proto_lib().flock_verify_chain(ctx.handle, buf.ctypes.data_as(ctypes.c_void_p), buf.size,
                                          _domain_bytes(domain),
                                          ctypes.byref(ok)), "flock_verify_chain")
    return bool(ok.value)


def chain_inputs(steps, seed, cv0=None):
    """Honest BLAKE3 chain as the flock_chain CLI builds it (host, sequential):
    records whose cv is the previous record's compression output."""
    out = np.zeros(steps, COMPRESSION_DTYPE)
    c = None if cv0 is None else np.ascontiguousarray(cv0, dtype=np.uint32)
    check(_proto_lib().flock_chain_inputs(steps, seed, None if c is None else c.ctypes.data_as(ctypes.c_void_p),
                                          out.ctypes.data_as(ctypes.c_void_p)), "flock_chain_inputs")
    return out
