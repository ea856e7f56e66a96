// Full proof orchestration on one GPU.
//
// Follows Blake3Setup::prove_fast (crates/flock-prover/src/r1cs_hashes/blake3.rs:3405-3642)
// and prove_ligerito (crates/flock-prover/src/prover.rs:194-289): witness ->
// PCS commit -> bind_statement -> zerocheck -> lincheck -> ring switch of the
// [ab, c] claims -> recursive Ligerito opening -> wire bytes
// (crates/flock-prover/src/proof_io.rs:161-208). All bulk work runs in the
// kernels of this library; the host keeps the Fiat-Shamir transcript and the
// O(1)-sized algebra between rounds (Lagrange weights, 64/128-entry vectors).
#include <algorithm>
#include <array>
#include <chrono>
#include <cstring>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "flock_internal.h"
#include "host_field.h"
#include "prover.h"
#include "r1cs_setup.h"
#include "transcript.h"
#include "zc_tables.h"

namespace {

using hf::F;

#include "ligerito_params.inc"

struct LigCfg {
  int initial_k = 0, yr_log_n = 0, steps = 0;
  std::vector<int> rates, ks, queries, grind_bits, fold_bits, ood;
};

bool lig_config(int m, int profile, LigCfg& c) {
  for (int i = 0; i < LIGERITO_N_CONFIGS; i++) {
    const int* row = LIGERITO_CONFIGS[i];
    if (row[0] != m || row[1] != profile) continue;
    c = LigCfg();
    c.initial_k = row[2];
    c.yr_log_n = row[3];
    int nl = row[4];
    c.steps = nl - 1;
    for (int l = 0; l < nl; l++) {
      const int* L = row + 5 + 8 * l;
      c.rates.push_back(L[0]);
      if (l > 0) c.ks.push_back(L[3]);
      c.queries.push_back(L[4]);
      c.grind_bits.push_back(L[5]);
      c.fold_bits.push_back(L[6]);
      c.ood.push_back(L[7]);
    }
    return true;
  }
  return false;
}

struct Fail : std::runtime_error {
  int code;
  Fail(int c, const std::string& w) : std::runtime_error(w), code(c) {}
};
// A CUDA status as a failure: a bounded wait that gave up (cudaErrorTimeout,
// from flock_stream_wait under a wait limit) is FLOCK_ERR_TIMEOUT.
#define CK(x)                                                                                            \
  do {                                                                                                   \
    cudaError_t e_ = (x);                                                                                \
    if (e_ != cudaSuccess)                                                                               \
      throw Fail(e_ == cudaErrorTimeout ? FLOCK_ERR_TIMEOUT : FLOCK_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)
#define FK(x)                                      \
  do {                                             \
    int r_ = (x);                                  \
    if (r_ != FLOCK_OK) throw Fail(r_, #x);        \
  } while (0)

struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void* get(size_t b) {
    if (b > bytes) {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      if (cudaMalloc(&p, b) != cudaSuccess) throw Fail(FLOCK_ERR_OOM, "cudaMalloc");
      bytes = b;
    }
    return p;
  }
};

inline int ilog2(size_t n) {
  int l = 0;
  while (((size_t)1 << l) < n) l++;
  return l;
}

// ---------------------------------------------------------------- host algebra
std::vector<F> eq_table(const std::vector<F>& r) {
  std::vector<F> t((size_t)1 << r.size());
  t[0] = F::one();
  for (size_t i = 0; i < r.size(); i++) {
    size_t h = (size_t)1 << i;
    for (size_t j = 0; j < h; j++) {
      F vr = t[j] * r[i];
      t[j + h] = vr;
      t[j] = t[j] + vr;
    }
  }
  return t;
}

// Lagrange weights on 64 nodes phi8(off..off+63) (multilinear.rs:361-520),
// prefix/suffix products with cached denominators.
struct Lagrange {
  std::vector<F> den_inv[2];
  Lagrange() {
    for (int k = 0; k < 2; k++) {
      den_inv[k].resize(64);
      for (int i = 0; i < 64; i++) {
        F si = hf::phi8((uint8_t)(64 * k + i)), d = F::one();
        for (int j = 0; j < 64; j++)
          if (j != i) d = d * (si + hf::phi8((uint8_t)(64 * k + j)));
        den_inv[k][i] = hf::inv(d);
      }
    }
  }
  std::vector<F> at(F z, int which) const {
    std::vector<F> w(64);
    F pre = F::one();
    for (int i = 0; i < 64; i++) {
      w[i] = pre;
      pre = pre * (z + hf::phi8((uint8_t)(64 * which + i)));
    }
    F suf = F::one();
    for (int i = 63; i >= 0; i--) {
      w[i] = w[i] * suf * den_inv[which][i];
      suf = suf * (z + hf::phi8((uint8_t)(64 * which + i)));
    }
    return w;
  }
};
const Lagrange& lagrange() {
  static const Lagrange L;
  return L;
}

// phi8(M[i][s]) for the S -> Lambda extension matrix, cached.
const std::vector<F>& phi_ext_matrix() {
  static const std::vector<F> pm = [] {
    auto M = zc::ext_matrix();
    std::vector<F> v(64 * 64);
    for (int i = 0; i < 64 * 64; i++) v[i] = hf::phi8(M[i]);
    return v;
  }();
  return pm;
}

F dot(const F* a, const F* b, size_t n) {
  F s;
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

std::vector<F> transpose128(const std::vector<F>& v) {
  std::vector<F> u(128);
  for (int i = 0; i < 128; i++)
    for (int b = 0; b < 128; b++) {
      uint64_t bit = b < 64 ? (v[i].lo >> b) & 1 : (v[i].hi >> (b - 64)) & 1;
      if (bit) {
        if (i < 64) u[b].lo |= 1ULL << i;
        else u[b].hi |= 1ULL << (i - 64);
      }
    }
  return u;
}

// s_k(v_k) and inverses, ligerito.rs:1747-1774.
struct Sks {
  std::vector<F> s, inv;
  std::vector<F> lin;  // [n][32]: What_k(x^b) for the bits b of a 32-bit index
};
const Sks& sks_for(int n) {
  static std::vector<Sks> cache(64);
  static std::vector<bool> have(64, false);
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  if (!have[n]) {
    Sks r;
    r.s.assign(n + 1, F());
    r.s[0] = F::one();
    std::vector<F> layer;
    for (int i = 1; i <= n; i++) layer.push_back(F(1ULL << i, 0));
    int cur = n;
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < cur; j++) {
        F v = layer[j] * layer[j] + r.s[i] * layer[j];
        if (j == 0) r.s[i + 1] = v;
        else layer[j - 1] = v;
      }
      cur--;
    }
    for (auto& v : r.s) r.inv.push_back(v.zero() ? F() : hf::inv(v));
    // s_k is GF(2)-linear: What_k(q) = sum over the set bits b of q of What_k(x^b)
    r.lin.assign((size_t)n * 32, F());
    for (int b = 0; b < 32; b++) {
      F s(1ULL << b, 0);
      for (int k = 0; k < n; k++) {
        if (k > 0) s = s * s + r.s[k - 1] * s;
        r.lin[(size_t)k * 32 + b] = s * r.inv[k];
      }
    }
    cache[n] = r;
    have[n] = true;
  }
  return cache[n];
}

std::vector<uint32_t> sample_queries(fs::Transcript& tr, size_t block_len, size_t count) {
  std::set<uint32_t> seen;
  std::vector<uint32_t> out;
  while (out.size() < count) {
    F v = tr.sample();
    uint32_t q = (uint32_t)(v.lo % block_len);
    if (seen.insert(q).second) out.push_back(q);
  }
  std::sort(out.begin(), out.end());
  return out;
}

// Node indices of the octopus multi-proof (crates/flock-core/src/merkle.rs:879-928)
// in emission order, for sorted unique positions.
std::vector<uint32_t> multiproof_nodes(size_t n_leaves, const std::vector<uint32_t>& pos) {
  std::vector<uint32_t> out;
  if (pos.empty() || n_leaves == 1) return out;
  std::vector<uint32_t> act(pos);
  size_t ls = 0, ll = n_leaves;
  while (ll > 1) {
    std::vector<uint32_t> nxt;
    size_t i = 0;
    while (i < act.size()) {
      uint32_t p = act[i];
      bool sib = i + 1 < act.size() && act[i + 1] == (p ^ 1u);
      if (sib) i += 2;
      else {
        out.push_back((uint32_t)(ls + (p ^ 1u)));
        i += 1;
      }
      nxt.push_back(p >> 1);
    }
    act.swap(nxt);
    ls += ll;
    ll >>= 1;
  }
  return out;
}

// ---------------------------------------------------------------- wire writer
struct Wire {
  std::vector<uint8_t> v;
  void raw(const void* p, size_t n) { v.insert(v.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void u32(uint32_t x) { raw(&x, 4); }
  void u64(uint64_t x) { raw(&x, 8); }
  void f(F x) { u64(x.lo); u64(x.hi); }
  void fv(const F* p, size_t n) { u64(n); raw(p, 16 * n); }
  void fv(const std::vector<F>& x) { fv(x.data(), x.size()); }
  void pv(const std::vector<std::pair<F, F>>& x) {
    u64(x.size());
    for (auto& e : x) { f(e.first); f(e.second); }
  }
};

struct Open {
  std::vector<F> rows;  // q x width
  size_t width = 0;
  std::vector<uint8_t> nodes;  // 32-byte hashes
  // Copied into the pinned openings area by the stream (no wait of its own):
  // rows and nodes are filled from there by finish_open once a later wait
  // has passed. -1: already filled.
  ptrdiff_t pin_rows = -1, pin_nodes = -1;
};

}  // namespace

// ============================================================================
constexpr int kSklMax = 40;  // induced-basis variable counts below this
constexpr int kKernelSpans = 4;  // witness, L0 NTT, L0 Merkle tree, zerocheck round 1

struct ProverState {
  int device = 0;
  cudaStream_t st = nullptr;  // the stream in use: st_normal or st_high
  cudaStream_t st_normal = nullptr, st_high = nullptr;
  ZcRound1Tables* d_r1t = nullptr;
  DBuf in, z, a, b, stripe, cw, tree, A0, B0, A1, B1, eqlo, eqhi, eqout, rdev, part, red, lag, small, eqin, comb,
      zvec, zvec0, tlo0, thi0, tlo1, thi1, tables, bc, f1, b1, W, LO, HI, basis, qbuf, abuf, rows, nidx, nodes,
      grind, lvl_cw[2], lvl_tree[2], chW, chG, zceq, zcr, zcjobs;
  DBuf csc_ap, csc_ai, csc_bp, csc_bi;
  bool csc_ready = false;
  DBuf skl[kSklMax];  // What_k(x^b) tables of the induced basis, per number of variables
  FlockPhaseTimes times;
  // Optional CUDA-event timing of the main kernels of a proof, on the
  // prover's stream: pairs of events around each span of kKernelSpans.
  bool timing = false;
  cudaEvent_t tev[2 * kKernelSpans] = {};
  float span_ms[kKernelSpans] = {};
  void mark(int i) {
    if (timing && tev[i]) cudaEventRecord(tev[i], st);
  }
  // Pinned host staging: small host->device copies are bump-allocated in
  // [0, kPinH2D) for the duration of one proof (pinned sources keep the
  // copies asynchronous); device->host reads go through the last kPinD2H bytes.
  uint8_t* pin = nullptr;
  size_t pin_off = 0;
  // Pinned area the opened rows and Merkle nodes of a proof are copied into
  // (bump-allocated per proof): they are only serialized at the end of the
  // proof, so their copies ride on the stream and need no wait of their own.
  uint8_t* pin_open = nullptr;
  size_t pin_open_off = 0;
  // Mapped pinned area for round partials: kernels write them straight into
  // host memory, so reading a round's message needs only the stream sync.
  uint8_t* mapped = nullptr;
  void* mapped_dev = nullptr;
  // The host's waits for the stream (flock_stream_wait) in the current proof.
  WaitStats waits;

  std::vector<DBuf*> bufs() {
    std::vector<DBuf*> v = {&in, &z, &a, &b, &stripe, &cw, &tree, &A0, &B0, &A1, &B1, &eqlo, &eqhi, &eqout, &rdev, &part, &red,
            &lag, &small, &eqin, &comb, &zvec, &zvec0, &tlo0, &thi0, &tlo1, &thi1, &tables, &bc, &f1, &b1,
            &W, &LO, &HI, &basis, &qbuf, &abuf, &rows, &nidx, &nodes, &grind, &lvl_cw[0], &lvl_cw[1],
            &lvl_tree[0], &lvl_tree[1], &chW, &chG, &zceq, &zcr, &zcjobs, &csc_ap, &csc_ai, &csc_bp, &csc_bi};
    for (DBuf& d : skl) v.push_back(&d);
    return v;
  }
  std::vector<const DBuf*> bufs() const {
    auto v = const_cast<ProverState*>(this)->bufs();
    return std::vector<const DBuf*>(v.begin(), v.end());
  }
};

namespace {

constexpr size_t kPinH2D = (size_t)4 << 20, kPinD2H = (size_t)1 << 20, kMapped = (size_t)256 << 10;
constexpr size_t kPinOpen = (size_t)4 << 20;
// Zerocheck rounds of at most this many pairs run on the host (see the round loop).
constexpr size_t kHostTailPairs = 512;
// Lincheck product-sumcheck rounds over at most this many entries run on the host.
constexpr size_t kHostTailLincheck = 1024;

void h2d(ProverState& S, void* d, const void* h, size_t n) {
  if (n == 0) return;
  const size_t need = (n + 255) & ~(size_t)255;
  if (S.pin && S.pin_off + need <= kPinH2D) {
    uint8_t* p = S.pin + S.pin_off;
    S.pin_off += need;
    std::memcpy(p, h, n);
    CK(cudaMemcpyAsync(d, p, n, cudaMemcpyHostToDevice, S.st));
  } else {
    CK(cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, S.st));
  }
}
void d2h(ProverState& S, void* h, const void* d, size_t n) {
  if (n == 0) return;
  if (S.pin && n <= kPinD2H) {
    uint8_t* p = S.pin + kPinH2D;
    CK(cudaMemcpyAsync(p, d, n, cudaMemcpyDeviceToHost, S.st));
    CK(flock_stream_wait(S.st, &S.waits));
    std::memcpy(h, p, n);
  } else {
    CK(cudaMemcpyAsync(h, d, n, cudaMemcpyDeviceToHost, S.st));
    CK(flock_stream_wait(S.st, &S.waits));
  }
}
// Two device->host reads behind one wait.
void d2h2(ProverState& S, void* h1, const void* d1, size_t n1, void* h2, const void* d2, size_t n2) {
  const size_t off2 = (n1 + 255) & ~(size_t)255;
  if (!S.pin || off2 + n2 > kPinD2H) {
    d2h(S, h1, d1, n1);
    d2h(S, h2, d2, n2);
    return;
  }
  uint8_t* p = S.pin + kPinH2D;
  if (n1) CK(cudaMemcpyAsync(p, d1, n1, cudaMemcpyDeviceToHost, S.st));
  if (n2) CK(cudaMemcpyAsync(p + off2, d2, n2, cudaMemcpyDeviceToHost, S.st));
  CK(flock_stream_wait(S.st, &S.waits));
  if (n1) std::memcpy(h1, p, n1);
  if (n2) std::memcpy(h2, p + off2, n2);
}
void u2(const F& x, uint64_t out[2]) { out[0] = x.lo; out[1] = x.hi; }

struct Clock {
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  double lap() {
    auto n = std::chrono::steady_clock::now();
    double ms = std::chrono::duration<double, std::milli>(n - t).count();
    t = n;
    return ms;
  }
};

// Ligero commit of poly (device, length 2^(lmc+lni)) into (cw, tree); returns root.
void ligero_commit(ProverState& S, const void* poly, int lmc, int lni, int rate, void* cw, void* tree,
                   uint8_t root[32]) {
  int log_d = lmc + rate;
  FK(flock_launch_ntt(cw, poly, log_d, lni, rate, S.st));
  size_t leaves = (size_t)1 << log_d;
  FK(flock_launch_merkle(cw, leaves, (size_t)16 << lni, tree, S.st));
  d2h(S, root, (const uint8_t*)tree + (2 * leaves - 2) * 32, 32);
}

Open open_rows(ProverState& S, const void* cw, const void* tree, size_t block_len, int width,
               const std::vector<uint32_t>& q) {
  Open o;
  o.width = width;
  uint32_t* dq = (uint32_t*)S.qbuf.get(q.size() * 4);
  h2d(S, dq, q.data(), q.size() * 4);
  void* dr = S.rows.get(q.size() * width * 16);
  FK(flock_launch_gather_rows(cw, dq, (int)q.size(), width, dr, S.st));
  // both gathers are queued before the first read: one wait for the two
  auto idx = multiproof_nodes(block_len, q);
  void* dn = nullptr;
  if (!idx.empty()) {
    uint32_t* di = (uint32_t*)S.nidx.get(idx.size() * 4);
    h2d(S, di, idx.data(), idx.size() * 4);
    dn = S.nodes.get(idx.size() * 32);
    FK(flock_launch_gather_nodes(tree, di, (int)idx.size(), dn, S.st));
  }
  o.rows.resize(q.size() * width);
  o.nodes.resize(idx.size() * 32);
  const size_t nr = o.rows.size() * 16, nn = dn ? o.nodes.size() : 0;
  const size_t need = ((nr + 255) & ~(size_t)255) + ((nn + 255) & ~(size_t)255);
  if (S.pin_open && S.pin_open_off + need <= kPinOpen) {
    o.pin_rows = (ptrdiff_t)S.pin_open_off;
    o.pin_nodes = (ptrdiff_t)(S.pin_open_off + ((nr + 255) & ~(size_t)255));
    S.pin_open_off += need;
    if (nr) CK(cudaMemcpyAsync(S.pin_open + o.pin_rows, dr, nr, cudaMemcpyDeviceToHost, S.st));
    if (nn) CK(cudaMemcpyAsync(S.pin_open + o.pin_nodes, dn, nn, cudaMemcpyDeviceToHost, S.st));
  } else {
    d2h2(S, o.rows.data(), dr, nr, o.nodes.data(), dn, nn);
  }
  return o;
}

// Fills an opening whose copies were queued by open_rows; the caller has
// waited for the stream since.
void finish_open(ProverState& S, Open& o) {
  if (o.pin_rows < 0) return;
  if (!o.rows.empty()) std::memcpy(o.rows.data(), S.pin_open + o.pin_rows, o.rows.size() * 16);
  if (!o.nodes.empty()) std::memcpy(o.nodes.data(), S.pin_open + o.pin_nodes, o.nodes.size());
  o.pin_rows = o.pin_nodes = -1;
}

void write_open(Wire& w, const Open& o) {
  size_t nq = o.width ? o.rows.size() / o.width : 0;
  w.u64(nq);
  for (size_t i = 0; i < nq; i++) w.fv(&o.rows[i * o.width], o.width);
  w.u64(o.nodes.size() / 32);
  w.raw(o.nodes.data(), o.nodes.size());
}

// Reduce `count` partial rows of `width` F128 on the device, copy to host.
// Reduce `count` partial rows of `width` F128 (XOR), result on the host. Up to
// 64 KiB of partials are copied and reduced on the host (one transfer instead
// of a reduction launch plus a transfer on the round's critical path); wider
// ones are reduced on the device first.
std::vector<F> reduce_partials(ProverState& S, const void* part, size_t count, int width) {
  std::vector<F> out(width);
  if (S.mapped && part == S.mapped_dev) {  // written by the kernel into host memory
    CK(flock_stream_wait(S.st, &S.waits));
    const F* rows = reinterpret_cast<const F*>(S.mapped);
    for (size_t c = 0; c < count; c++)
      for (int k = 0; k < width; k++) out[k] += rows[c * width + k];
    return out;
  }
  if (count * (size_t)width <= 4096) {
    std::vector<F> rows(count * (size_t)width);
    d2h(S, rows.data(), part, rows.size() * 16);
    for (size_t c = 0; c < count; c++)
      for (int k = 0; k < width; k++) out[k] += rows[c * width + k];
    return out;
  }
  void* r = S.red.get((size_t)width * 16);
  FK(flock_launch_reduce_rows(part, count, width, r, S.st));
  d2h(S, out.data(), r, (size_t)width * 16);
  return out;
}

// Partials buffer of a round: the mapped host area when it fits (one round
// at a time: reduce_partials reads it before the next round is launched).
void* part_buf(ProverState& S, size_t bytes) {
  if (S.mapped && bytes <= kMapped) return S.mapped_dev;
  return S.part.get(bytes);
}

void eq_split_dev(ProverState& S, const std::vector<F>& r, int lo_bits, DBuf& lo, DBuf& hi) {
  int hi_bits = (int)r.size() - lo_bits;
  void* dr = S.rdev.get(r.size() * 16 + 16);
  h2d(S, dr, r.data(), r.size() * 16);
  FK(flock_launch_eq_split(dr, lo_bits, hi_bits, lo.get((size_t)16 << lo_bits), hi.get((size_t)16 << hi_bits), S.st));
}

}  // namespace

ProverState* flock_prover_create(int device) {
  ProverState* S = new ProverState;
  S->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&S->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete S;
    return nullptr;
  }
  S->st_normal = S->st;
  // the high-priority stream (flock_prover_set_priority); without one, the
  // prover keeps its normal stream
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
      cudaStreamCreateWithPriority(&S->st_high, cudaStreamNonBlocking, greatest) != cudaSuccess)
    S->st_high = nullptr;
  cudaGetLastError();
  // Without pinned staging the copies still work, through the driver's own.
  void* pin = nullptr;
  if (cudaMallocHost(&pin, kPinH2D + kPinD2H) == cudaSuccess) S->pin = (uint8_t*)pin;
  else cudaGetLastError();
  void* po = nullptr;
  if (cudaMallocHost(&po, kPinOpen) == cudaSuccess) S->pin_open = (uint8_t*)po;
  else cudaGetLastError();
  void* m = nullptr;
  if (cudaHostAlloc(&m, kMapped, cudaHostAllocMapped) == cudaSuccess) {
    if (cudaHostGetDevicePointer(&S->mapped_dev, m, 0) == cudaSuccess) S->mapped = (uint8_t*)m;
    else cudaFreeHost(m);
  }
  cudaGetLastError();
  return S;
}

void flock_prover_destroy(ProverState* S) {
  if (!S) return;
  cudaSetDevice(S->device);
  for (cudaEvent_t e : S->tev)
    if (e) cudaEventDestroy(e);
  if (S->d_r1t) cudaFree(S->d_r1t);
  if (S->st_normal) cudaStreamDestroy(S->st_normal);
  if (S->st_high) cudaStreamDestroy(S->st_high);
  if (S->pin) cudaFreeHost(S->pin);
  if (S->pin_open) cudaFreeHost(S->pin_open);
  if (S->mapped) cudaFreeHost(S->mapped);
  delete S;
}

size_t flock_prover_reserved_bytes(const ProverState* S) {
  size_t t = S->d_r1t ? sizeof(ZcRound1Tables) : 0;
  for (const DBuf* b : S->bufs()) t += b->bytes;
  return t;
}

void flock_prover_trim(ProverState* S) {
  cudaSetDevice(S->device);
  cudaStreamSynchronize(S->st);
  for (DBuf* b : S->bufs()) b->release();
  S->csc_ready = false;
}

const FlockPhaseTimes& flock_prover_times(const ProverState* S) { return S->times; }

int flock_prover_set_wait_limit(ProverState* S, double limit_ms) {
  if (!(limit_ms >= 0)) return FLOCK_ERR_ARG;  // NaN included
  S->waits.limit_ms = limit_ms;
  return FLOCK_OK;
}

int flock_prover_set_timing(ProverState* S, bool on) {
  if (on) {
    if (cudaSetDevice(S->device) != cudaSuccess) return FLOCK_ERR_CUDA;
    for (cudaEvent_t& e : S->tev)
      if (!e && cudaEventCreate(&e) != cudaSuccess) return FLOCK_ERR_CUDA;
  }
  S->timing = on;
  return FLOCK_OK;
}

int flock_prover_kernel_times(const ProverState* S, double* ms, int n) {
  for (int k = 0; k < n && k < kKernelSpans; k++) ms[k] = S->timing ? S->span_ms[k] : 0.0;
  return FLOCK_OK;
}
cudaStream_t flock_prover_stream(const ProverState* S) { return S->st; }

void flock_prover_set_priority(ProverState* S, bool high) {
  cudaStream_t want = high && S->st_high ? S->st_high : S->st_normal;
  if (want == S->st) return;
  cudaSetDevice(S->device);
  cudaStreamSynchronize(S->st);  // the previous proof's work is done before its buffers change streams
  S->st = want;
}

int flock_prover_prove_seed(ProverState* S, int log2, uint64_t seed, std::vector<uint8_t>& out) {
  try {
    CK(cudaSetDevice(S->device));
    size_t n = (size_t)1 << log2;
    uint64_t l = (uint64_t)log2;
    uint64_t state0 = seed ^ ((l << 29) | (l >> 35));
    void* d_in = S->in.get(n * sizeof(flock_compression));
    FK(flock_launch_gen_inputs(state0, n, d_in, S->st));
    int n_log = log2 < 3 ? 3 : log2;
    return flock_prover_prove(S, (const flock_compression*)d_in, n, n_log, out, true);
  } catch (const Fail& f) {
    return f.code;
  }
}

int flock_prover_prove(ProverState* S, const flock_compression* h_in, size_t n, int n_log, std::vector<uint8_t>& out,
                       bool input_on_device, const ChainReq* chain, fs::Transcript* ext_tr, flock_r1cs_claim* claim) {
  try {
    CK(cudaSetDevice(S->device));
    // the staging area of the previous call is free again (under a wait
    // limit, this also drains the work of a call that gave up waiting)
    CK(flock_stream_wait(S->st, &S->waits, false));
    S->pin_off = 0;
    S->pin_open_off = 0;
    const int m = 14 + n_log;
    LigCfg cfg;
    if (!lig_config(m, 0, cfg)) return FLOCK_ERR_SHAPE;
    if (n > ((size_t)1 << n_log) || n_log < 8) return FLOCK_ERR_SHAPE;
    // the chain shift relation covers every slot: the steps must fill 2^n_log
    if (chain && n != ((size_t)1 << n_log)) return FLOCK_ERR_SHAPE;
    cudaStream_t st = S->st;
    FlockPhaseTimes& T = S->times;
    T = FlockPhaseTimes();
    S->waits.waits = 0;  // counted per proof; the wait limit stays
    S->waits.blocked_ms = 0;
    uint64_t waits_seen = 0;
    double blocked_seen = 0;
    auto snap_waits = [&](int phase) {
      T.waits[phase] = S->waits.waits - waits_seen;
      T.blocked_ms[phase] = S->waits.blocked_ms - blocked_seen;
      waits_seen = S->waits.waits;
      blocked_seen = S->waits.blocked_ms;
    };
    Clock clk;
    // ---- setup constants (cached) ----
    uint8_t digest[32];
    flock_statement_digest(m, digest);
    if (!S->d_r1t) {
      ZcRound1Tables* h = new ZcRound1Tables;
      zc::build_round1_tables(*h);
      CK(cudaMalloc(&S->d_r1t, sizeof(ZcRound1Tables)));
      CK(cudaMemcpy(S->d_r1t, h, sizeof(ZcRound1Tables), cudaMemcpyHostToDevice));
      delete h;
    }
    if (!S->csc_ready) {
      const HostCsc& c = flock_host_csc();
      h2d(*S, S->csc_ap.get(c.a_ptr.size() * 4), c.a_ptr.data(), c.a_ptr.size() * 4);
      h2d(*S, S->csc_ai.get(c.a_idx.size() * 4), c.a_idx.data(), c.a_idx.size() * 4);
      h2d(*S, S->csc_bp.get(c.b_ptr.size() * 4), c.b_ptr.data(), c.b_ptr.size() * 4);
      h2d(*S, S->csc_bi.get(c.b_idx.size() * 4), c.b_idx.data(), c.b_idx.size() * 4);
      CK(flock_stream_wait(st, &S->waits, false));
      S->csc_ready = true;
    }
    const Lagrange& LG = lagrange();
    T.setup_ms = clk.lap();
    snap_waits(0);

    // ---- witness + commit ----
    const size_t nbits = (size_t)1 << m, nbytes = nbits / 8, n128 = nbits / 128;
    const void* d_in = h_in;
    if (!input_on_device) {
      void* buf = S->in.get(std::max<size_t>(n, 1) * sizeof(flock_compression));
      if (n) h2d(*S, buf, h_in, n * sizeof(flock_compression));
      d_in = buf;
    }
    void *dz = S->z.get(nbytes), *da = S->a.get(nbytes), *db = S->b.get(nbytes), *ds = S->stripe.get(nbytes);
    S->mark(0);
    FK(flock_launch_witness((const flock_compression*)d_in, n, n_log, dz, da, db, ds, st));
    S->mark(1);
    const int lbs = 6, rate0 = 1;
    const int log_d0 = m - 7 - lbs + rate0;
    const size_t block0 = (size_t)1 << log_d0;
    void* dcw = S->cw.get((n128 << rate0) * 16);
    void* dtree = S->tree.get((2 * block0 - 1) * 32);
    S->mark(2);
    FK(flock_launch_ntt(dcw, dz, log_d0, lbs, rate0, st));
    S->mark(3);
    S->mark(4);
    FK(flock_launch_merkle(dcw, block0, (size_t)16 << lbs, dtree, st));
    S->mark(5);
    uint8_t root0[32];
    d2h(*S, root0, (const uint8_t*)dtree + (2 * block0 - 2) * 32, 32);
    T.commit_ms = clk.lap();
    snap_waits(1);

    Wire w;
    w.raw("FLOCK", 5);
    uint8_t ver[2] = {4, (uint8_t)(chain ? 3 : 2)};  // flavor 2 = R1CS, 3 = chain (proof_io.rs:8-13)
    w.raw(ver, 2);
    if (chain) w.u32(0);  // HashKind::Blake3 of the chain bundle
    w.raw(root0, 32);
    w.u64(m);
    w.u64(rate0);
    w.u64(lbs);
    w.u32(0);  // LigeritoProfile::Fast
    w.u32(1);  // HashKind::Blake3

    // the caller's transcript is copied and written back only when the proof is made
    fs::Transcript tr = ext_tr ? *ext_tr : fs::Transcript(chain ? chain->domain : "flock-bench-v0");
    // bind_statement (crates/flock-core/src/proof.rs:51-59)
    tr.label("flock-r1cs-v0");
    tr.observe_bytes(digest, 32);
    tr.observe_bytes(root0, 32);

    // ---- zerocheck ----
    tr.label("flock-zerocheck-v0");
    std::vector<F> r(m);
    {
      auto rs = tr.sample_vec(6);
      auto ro = tr.sample_vec(m - 13);
      for (int i = 0; i < 6; i++) r[i] = rs[i];
      for (int i = 0; i < 3; i++) r[6 + i] = hf::phi8(zc::SMALL_CHAL[i]);
      for (int i = 0; i < 4; i++) {
        F g(1ULL << (1 << i), 0);
        r[9 + i] = g * hf::inv(F::one() + g);
      }
      for (int i = 13; i < m; i++) r[i] = ro[i - 13];
    }
    std::vector<F> p_ab(64), p_c(64), shv_c;
    {
      const size_t rows = nbits / 64, n_outer = rows / 128;
      std::vector<F> rout(r.begin() + 13, r.end());
      int nv = (int)rout.size();
      void* dr = S->rdev.get(rout.size() * 16 + 16);
      h2d(*S, dr, rout.data(), rout.size() * 16);
      // eq_out, then round 1's per-block table basis phi8(2^k) eq_out(xo)
      // behind it in the same buffer
      void* deq = S->eqout.get(n_outer * 16 * 9);
      void* dbasis = (uint8_t*)deq + n_outer * 16;
      FK(flock_launch_eq_split(dr, nv, 0, deq, S->eqhi.get(16), st));
      FK(flock_launch_zc1_eq_basis(deq, n_outer, S->d_r1t, dbasis, st));
      const int grid = 152;
      void* dpart = S->part.get((size_t)grid * 192 * 16);
      S->mark(6);
      FK(flock_launch_zc_round1(da, db, dz, n_outer, dbasis, S->d_r1t, dpart, grid, st));
      S->mark(7);
      auto sums = reduce_partials(*S, dpart, grid, 192);
      F dinv = zc::medium_dinv();
      const std::vector<F>& PM = phi_ext_matrix();
      // S[64t + s] (ring-switch statistic of the c claim) and C_s = (1 + r6) S[s] + r6 S[64 + s]
      shv_c.resize(128);
      for (int b2 = 0; b2 < 128; b2++) shv_c[b2] = dinv * sums[64 + b2];
      std::vector<F> cs(64);
      for (int s = 0; s < 64; s++) cs[s] = (F::one() + r[6]) * shv_c[s] + r[6] * shv_c[64 + s];
      for (int i = 0; i < 64; i++) {
        p_ab[i] = dinv * sums[i];
        p_c[i] = dot(&PM[i * 64], cs.data(), 64);
      }
    }
    T.zc_round1_ms = clk.lap();
    snap_waits(2);
    tr.observe_slice(p_ab.data(), 64);
    tr.observe_slice(p_c.data(), 64);
    F zc_z = tr.sample();
    F final_c;
    {
      auto wl = LG.at(zc_z, 1);
      final_c = dot(wl.data(), p_c.data(), 64);
    }
    auto lag_z = LG.at(zc_z, 0);
    const size_t rows0 = nbits / 64;
    void *dA0 = S->A0.get(rows0 * 16), *dB0 = S->B0.get(rows0 * 16);
    void *dA1 = S->A1.get(rows0 / 2 * 16), *dB1 = S->B1.get(rows0 / 2 * 16);
    void* dlag = S->lag.get(64 * 16);
    h2d(*S, dlag, lag_z.data(), 64 * 16);
    const int n_mlv = m - 6;
    std::vector<std::pair<F, F>> zc_rounds;
    std::vector<F> rho;
    void *curA = dA0, *curB = dB0, *nxtA = dA1, *nxtB = dB1;
    // r[9..12] = g / (1 + g), g = x^(2^(k-9)): eq(r_k, b) = (1 + r_k) x^(b 2^(k-9))
    auto shift_var = [&](int k) { return (F::one() + r[k]) * F(1ULL << (1 << (k - 9)), 0) == r[k]; };
    // Per-round eq layout. The tables depend on r only, so all rounds' tables
    // are built by one launch before the first round (no eq work between a
    // round's kernel and the host's read of its message).
    struct RoundEq {
      bool grp;
      int a_bits, m_bits, f0, lob;
      F dinv;
      std::vector<F> vars;  // the variables of the split tables
    };
    auto round_eq = [&](int i) {
      std::vector<F> rr(r.begin() + 6 + i + 1, r.end());
      const int nv = (int)rr.size();
      // lowest variables of rr that are fixed challenges: phi8 ones (r7, r8)
      // and shift ones (r9..r12); rounds 0..5 factor their eq weight
      RoundEq q;
      q.a_bits = std::max(0, 2 - i);
      q.f0 = std::max(9, 7 + i);
      q.m_bits = std::max(0, 13 - q.f0);
      q.grp = q.m_bits > 0 && nv > q.a_bits + q.m_bits;
      for (int k = q.f0; q.grp && k < 13; k++) q.grp = shift_var(k);
      q.dinv = F::one();
      if (q.grp) {
        for (int k = q.f0; k < 13; k++) q.dinv = q.dinv * (F::one() + r[k]);
        std::vector<F> rg(rr.begin(), rr.begin() + q.a_bits);
        rg.insert(rg.end(), rr.begin() + q.a_bits + q.m_bits, rr.end());
        q.lob = std::min(nv - q.m_bits, 8);
        q.vars = std::move(rg);
      } else {
        // a CTA takes whole rows of 2^lob pairs: rows of 2^(nv - 10) pairs,
        // at least 2^8 (one pair per thread) and at most 2^12, keep the grid
        // near 608 CTAs while the round has pairs for it (rows of 2^12 left
        // rounds 7..13 on 1..64 CTAs, ~90 us each)
        q.lob = std::min(nv, std::max(8, std::min(12, nv - 10)));
        q.vars = std::move(rr);
      }
      return q;
    };
    std::vector<RoundEq> qs;
    std::vector<std::pair<size_t, size_t>> eq_off;  // (lo, hi) F128 offsets in zceq
    {
      std::vector<F> vars;
      std::vector<size_t> var_off;
      size_t tot = 0, max_entries = 0;
      for (int i = 0; i < n_mlv; i++) {
        qs.push_back(round_eq(i));
        const RoundEq& q = qs.back();
        const int hb = (int)q.vars.size() - q.lob;
        if (q.lob > 28 || hb > 28) throw Fail(FLOCK_ERR_SHAPE, "eq split");
        var_off.push_back(vars.size());
        vars.insert(vars.end(), q.vars.begin(), q.vars.end());
        eq_off.push_back({tot, tot + ((size_t)1 << q.lob)});
        tot += ((size_t)1 << q.lob) + ((size_t)1 << hb);
        max_entries = std::max(max_entries, ((size_t)1 << q.lob) + ((size_t)1 << hb));
      }
      F* dvars = (F*)S->zcr.get(vars.size() * 16 + 16);
      h2d(*S, dvars, vars.data(), vars.size() * 16);
      F* deq = (F*)S->zceq.get(tot * 16);
      std::vector<FlockEqJob> jobs(n_mlv);
      for (int i = 0; i < n_mlv; i++)
        jobs[i] = {dvars + var_off[i], deq + eq_off[i].first, deq + eq_off[i].second, qs[i].lob,
                   (int)qs[i].vars.size() - qs[i].lob};
      auto* djobs = (FlockEqJob*)S->zcjobs.get(jobs.size() * sizeof(FlockEqJob));
      h2d(*S, djobs, jobs.data(), jobs.size() * sizeof(FlockEqJob));
      FK(flock_launch_eq_split_multi(djobs, n_mlv, max_entries, st));
    }
    // The last rounds, from kHostTailPairs pairs down, run on the host: a GPU
    // round of a few hundred pairs is a latency-bound launch plus a round
    // trip (~20 us), the same round on the host a few microseconds.
    int host_from = n_mlv;
    while (host_from > 1 && (rows0 >> host_from) <= kHostTailPairs && !qs[host_from - 1].grp) host_from--;
    for (int i = 0; i < host_from; i++) {
      const size_t n_pairs = rows0 >> (i + 1);  // pairs of the round-i table
      const RoundEq& q = qs[i];
      const F* deq = (const F*)S->zceq.p;
      const void* elo = deq + eq_off[i].first;
      const void* ehi = deq + eq_off[i].second;
      uint64_t rp[2] = {0, 0};
      if (i > 0) u2(rho.back(), rp);
      int grid;
      void* dpart;
      if (q.grp) {
        grid = (int)std::min<size_t>(n_pairs >> (q.lob + q.m_bits), 152 * 4);
        dpart = part_buf(*S, (size_t)grid * 2 * 16);
        FK(flock_launch_zc_round_grp(i == 0 ? da : curA, i == 0 ? db : curB, n_pairs, i == 0, rp, dlag,
                                     i == 0 ? dA0 : nxtA, i == 0 ? dB0 : nxtB, elo, ehi, q.lob, q.a_bits, q.m_bits,
                                     1 << (q.f0 - 9), dpart, grid, st));
      } else {
        grid = (int)std::max<size_t>(std::min<size_t>(n_pairs >> q.lob, 152 * 4), 1);
        dpart = part_buf(*S, (size_t)grid * 2 * 16);
        if (i == 0)  // skip fold (multilinear.rs:598-630) fused into round 0
          FK(flock_launch_zc_round0_skip(da, db, n_pairs, dlag, dA0, dB0, elo, ehi, q.lob, dpart, grid, st));
        else
          FK(flock_launch_zc_round(curA, curB, n_pairs, 1, rp, nxtA, nxtB, elo, ehi, q.lob, dpart, grid, st));
      }
      auto g = reduce_partials(*S, dpart, grid, 2);
      g[0] = g[0] * q.dinv;
      g[1] = g[1] * q.dinv;
      if (i > 0) {
        std::swap(curA, nxtA);
        std::swap(curB, nxtB);
      }
      zc_rounds.push_back({g[0], g[1]});
      tr.observe(g[0]);
      tr.observe(g[1]);
      rho.push_back(tr.sample());
    }
    F fa, fb;
    if (host_from == n_mlv) {
      uint64_t rp[2];
      u2(rho.back(), rp);
      FK(flock_launch_bind_pairs(curA, curB, 1, rp, nxtA, nxtB, st));
      d2h(*S, &fa, nxtA, 16);
      d2h(*S, &fb, nxtB, 16);
    } else {
      // rounds host_from .. n_mlv - 1 on the host, from the table the last
      // GPU round wrote (2 entries per pair of that round, 4 per pair of round
      // host_from, which binds them at the last GPU round's challenge first),
      // as zc_round_kernel computes
      // them: bind A' = A0 + rho (A0 + A1), then G(1) = sum_j eq[j] a1 b1,
      // G(inf) = sum_j eq[j] (a0 + a1)(b0 + b1) over eq of the round's
      // remaining variables
      const size_t n_in = (rows0 >> host_from) * 2;
      std::vector<F> tA(n_in), tB(n_in);
      d2h(*S, tA.data(), curA, n_in * 16);
      d2h(*S, tB.data(), curB, n_in * 16);
      auto bind = [](std::vector<F>& v, F rr) {
        for (size_t j = 0; j < v.size() / 2; j++) v[j] = v[2 * j] + rr * (v[2 * j] + v[2 * j + 1]);
        v.resize(v.size() / 2);
      };
      for (int i = host_from; i < n_mlv; i++) {
        bind(tA, rho.back());
        bind(tB, rho.back());
        const std::vector<F> rr(r.begin() + 6 + i + 1, r.end());
        const std::vector<F> eq = eq_table(rr);
        F g1, gi;
        for (size_t j = 0; j < tA.size() / 2; j++) {
          const F a0 = tA[2 * j], a1 = tA[2 * j + 1], b0 = tB[2 * j], b1 = tB[2 * j + 1];
          g1 += eq[j] * (a1 * b1);
          gi += eq[j] * ((a0 + a1) * (b0 + b1));
        }
        g1 = g1 * qs[i].dinv;
        gi = gi * qs[i].dinv;
        zc_rounds.push_back({g1, gi});
        tr.observe(g1);
        tr.observe(gi);
        rho.push_back(tr.sample());
      }
      bind(tA, rho.back());
      bind(tB, rho.back());
      fa = tA[0];
      fb = tB[0];
    }
    tr.observe(fa);
    tr.observe(fb);
    T.zc_rounds_ms = clk.lap();
    snap_waits(3);
    w.fv(p_ab);
    w.fv(p_c);
    w.pv(zc_rounds);
    w.f(fa);
    w.f(fb);
    w.f(final_c);

    // ---- lincheck ----
    const int inner_rest = 14 - 6, n_outer_log = m - 14;
    std::vector<F> x_in(rho.begin(), rho.begin() + inner_rest), x_out(rho.begin() + inner_rest, rho.end());
    tr.label("flock-lincheck-v0");
    F alpha = tr.sample();
    F beta = tr.sample();
    std::vector<F> lc_rr;
    std::vector<std::pair<F, F>> lc_rounds;
    std::vector<F> z_partial(64);
    {
      void* dxr = S->small.get(inner_rest * 16);
      h2d(*S, dxr, x_in.data(), inner_rest * 16);
      void* deqin = S->eqin.get(FLOCK_K * 16);
      FK(flock_launch_lc_quirky_eq(dlag, dxr, inner_rest, deqin, st));
      void* dcomb = S->comb.get(FLOCK_K * 16);
      uint64_t al[2], be[2];
      u2(alpha, al);
      u2(beta, be);
      FK(flock_launch_lc_comb((const uint32_t*)S->csc_ap.p, (const uint32_t*)S->csc_ai.p, (const uint32_t*)S->csc_bp.p,
                              (const uint32_t*)S->csc_bi.p, deqin, al, be, 512, dcomb, st));
      int lob = n_outer_log / 2;
      eq_split_dev(*S, x_out, lob, S->eqlo, S->eqhi);
      size_t n_stripes = ((size_t)1 << n_outer_log) / 8;
      int grid = (int)std::min<size_t>(n_stripes / 8, 152);  // partial rows (stripe-group partitions)
      void* dpart = S->part.get((size_t)grid * FLOCK_K * 16);
      FK(flock_launch_lc_partial_fold(ds, n_stripes, S->eqlo.p, S->eqhi.p, lob, dpart, grid, st));
      void* dzv = S->zvec.get(FLOCK_K * 16);
      FK(flock_launch_reduce_rows(dpart, grid, FLOCK_K, dzv, st));
      CK(cudaMemcpyAsync(S->zvec0.get(FLOCK_K * 16), dzv, FLOCK_K * 16, cudaMemcpyDeviceToDevice, st));
      // product sumcheck on (comb, z_vec) binding the top variable
      // (lincheck.rs:1242-1300): the same round as the chain shift sumcheck
      // Rounds over at most kHostTailLincheck entries (and the final bind)
      // run on the host from the tables the last device round left, as
      // chain_round_kernel computes them: bind the top variable, then
      // q(1) = sum W_hi g_hi, q(inf) = sum (W_lo + W_hi)(g_lo + g_hi).
      size_t len = FLOCK_K;
      int t = 0;
      for (; t < inner_rest; t++) {
        if (t > 0 && (len / 2) <= kHostTailLincheck) break;
        uint64_t rp[2] = {0, 0};
        if (t > 0) u2(lc_rr.back(), rp);
        if (t > 0) len /= 2;
        const int grid = flock_chain_round_grid(len);
        void* dpart = part_buf(*S, (size_t)grid * 2 * 16);
        FK(flock_launch_chain_round(dcomb, dzv, len, t > 0, rp, dpart, grid, st));
        auto msg = reduce_partials(*S, dpart, grid, 2);
        tr.observe(msg[0]);
        tr.observe(msg[1]);
        lc_rounds.push_back({msg[0], msg[1]});
        lc_rr.push_back(tr.sample());
      }
      std::vector<F> hW(len), hg(len);  // the tables bound up to round t - 1 (2 x the next length)
      d2h(*S, hW.data(), dcomb, len * 16);
      d2h(*S, hg.data(), dzv, len * 16);
      auto bind_top = [](std::vector<F>& v, F rr) {
        const size_t h = v.size() / 2;
        for (size_t i = 0; i < h; i++) v[i] = v[i] + rr * (v[i + h] + v[i]);
        v.resize(h);
      };
      for (; t < inner_rest; t++) {
        bind_top(hW, lc_rr.back());
        bind_top(hg, lc_rr.back());
        const size_t q = hW.size() / 2;
        F e1, ei;
        for (size_t i = 0; i < q; i++) {
          e1 += hW[i + q] * hg[i + q];
          ei += (hW[i] + hW[i + q]) * (hg[i] + hg[i + q]);
        }
        tr.observe(e1);
        tr.observe(ei);
        lc_rounds.push_back({e1, ei});
        lc_rr.push_back(tr.sample());
      }
      // final bind to the 64 entries of z_partial
      bind_top(hW, lc_rr.back());
      bind_top(hg, lc_rr.back());
      std::copy(hg.begin(), hg.begin() + 64, z_partial.begin());
    }
    tr.observe_slice(z_partial.data(), 64);
    const F lc_skip = tr.sample();  // lincheck's skip challenge: the ab claim's z_skip
    std::vector<F> r_inner_rest(lc_rr.rbegin(), lc_rr.rend());
    if (claim) {
      // R1csClaim { ab, c } (crates/flock-prover/src/prover.rs:255-262), RowMajor
      // points (crates/flock-core/src/r1cs.rs:289-334): ab = (skip, r_inner_rest,
      // x_outer) with w = <Lagrange_S(skip), z_partial>; c = (zerocheck skip
      // point, r[6..14), r[14..m)) with the extracted c evaluation.
      std::memset(claim, 0, sizeof(*claim));
      const int n_out = m - 14;
      if (n_out > FLOCK_CLAIM_MAX_OUTER) throw Fail(FLOCK_ERR_SHAPE, "claim size");
      auto wl = LG.at(lc_skip, 0);
      u2(lc_skip, claim->ab.z_skip);
      u2(dot(wl.data(), z_partial.data(), 64), claim->ab.value);
      u2(zc_z, claim->c.z_skip);
      u2(final_c, claim->c.value);
      for (int i = 0; i < 8; i++) {
        u2(r_inner_rest[i], claim->ab.x_inner_rest[i]);
        u2(r[6 + i], claim->c.x_inner_rest[i]);
      }
      for (int i = 0; i < n_out; i++) {
        u2(x_out[i], claim->ab.x_outer[i]);
        u2(r[14 + i], claim->c.x_outer[i]);
      }
      claim->ab.n_outer = claim->c.n_outer = (uint32_t)n_out;
    }
    T.lincheck_ms = clk.lap();
    snap_waits(4);
    w.pv(lc_rounds);
    w.fv(z_partial);

    // ---- chain: region fold and shift sumcheck (chain_common.rs:316-320, chain.rs:155-233) ----
    std::vector<F> pd_inst;
    F pd_tau, pd_sel0, pd_value;
    if (chain) {
      pd_tau = tr.sample_vec(1)[0];
      const size_t N = (size_t)1 << n_log;
      void* dW = S->chW.get(2 * N * 16);
      void* dg = S->chG.get(2 * N * 16);
      uint64_t e0[2], e1[2];
      u2(F::one() + pd_tau, e0);
      u2(pd_tau, e1);
      FK(flock_launch_chain_fold_io(dz, N, e0, e1, dg, st));
      auto tau = tr.sample_vec(n_log);
      F al = tr.sample();
      int lob = std::min(n_log, 12);
      eq_split_dev(*S, tau, lob, S->eqlo, S->eqhi);
      uint64_t alu[2];
      u2(al, alu);
      FK(flock_launch_chain_weights(S->eqlo.p, S->eqhi.p, lob, N, alu, dW, st));
      std::vector<std::pair<F, F>> rounds;
      std::vector<F> rs;
      for (int k = 0; k <= n_log; k++) {
        const size_t h = (2 * N) >> k;
        int grid = flock_chain_round_grid(h);
        void* dpart = part_buf(*S, (size_t)grid * 2 * 16);
        uint64_t rp[2] = {0, 0};
        if (k > 0) u2(rs.back(), rp);
        FK(flock_launch_chain_round(dW, dg, h, k > 0, rp, dpart, grid, st));
        auto sm = reduce_partials(*S, dpart, grid, 2);
        tr.observe(sm[0]);
        tr.observe(sm[1]);
        rounds.push_back({sm[0], sm[1]});
        rs.push_back(tr.sample());
      }
      F g2[2];
      d2h(*S, g2, dg, 32);
      pd_value = g2[0] + rs.back() * (g2[1] + g2[0]);
      // round k bound coordinate n - k: instance coordinates are rs[n..1], the selector rs[0]
      pd_sel0 = rs[0];
      pd_inst.assign(rs.rbegin(), rs.rend() - 1);
      w.pv(rounds);
      w.f(pd_value);
    }

    // ---- PCS open: ring switch of [ab, c] (pcs.rs:1025-1110) ----
    tr.label("flock-pcs-open-batch-v0");
    std::vector<F> x_ab(r_inner_rest);
    x_ab.insert(x_ab.end(), x_out.begin(), x_out.end());
    std::vector<F> x_c(r.begin() + 6, r.end());
    const std::vector<F>* xs[2] = {&x_ab, &x_c};
    DBuf* tlo[2] = {&S->tlo0, &S->tlo1};
    DBuf* thi[2] = {&S->thi0, &S->thi1};
    std::vector<F> s_hat[2], eqr[2];
    F claims[2];
    const int L = m - 7;
    const int rs_lo = std::min(13, L - 1);
    {
      // ab claim: from the pre-sumcheck z_vec; c claim: from zerocheck round 1.
      std::vector<F> tail(r_inner_rest.begin() + 1, r_inner_rest.end());
      auto eq_tail = eq_table(tail);
      void* det = S->small.get(128 * 16);
      h2d(*S, det, eq_tail.data(), 128 * 16);
      void* dsh = S->red.get(128 * 16);
      FK(flock_launch_shv_from_zvec(S->zvec0.p, det, S->part.get(32 * 128 * 16), dsh, st));
      s_hat[0].resize(128);
      d2h(*S, s_hat[0].data(), dsh, 128 * 16);
      s_hat[1] = shv_c;
    }
    for (int k = 0; k < 2; k++) {
      tr.label("flock-ring-switch-v0");
      std::vector<F> suffix(xs[k]->begin() + 1, xs[k]->end());
      eq_split_dev(*S, suffix, rs_lo, *tlo[k], *thi[k]);
      tr.observe_slice(s_hat[k].data(), 128);
      auto rpp = tr.sample_vec(7);
      eqr[k] = eq_table(rpp);
      auto u = transpose128(s_hat[k]);
      claims[k] = dot(u.data(), eqr[k].data(), 128);
    }
    F gam[2] = {tr.sample(), tr.sample()};
    F target = gam[0] * claims[0] + gam[1] * claims[1];
    void* dbc = S->bc.get(n128 * 16);
    int msg0_grid = 0;  // > 0: the first Ligerito message's partials are in msg0_part
    void* msg0_part = nullptr;
    {
      // w_k[b] = gamma_k eq(r''_k)[b]: the basis is sum_k sum_b bit_b(t_k) w_k[b]
      std::vector<F> wk(2 * 128);
      for (int k = 0; k < 2; k++)
        for (int bb = 0; bb < 128; bb++) wk[k * 128 + bb] = gam[k] * eqr[k][bb];
      void* dt = S->tables.get(wk.size() * 16);
      h2d(*S, dt, wk.data(), wk.size() * 16);
      if (chain) {
        FK(flock_launch_combined_basis(n128, S->tlo0.p, S->thi0.p, S->tlo1.p, S->thi1.p, rs_lo, dt, dbc, st));
      } else {
        // the first Ligerito message over (z, b) comes out of the same pass;
        // nothing else writes the partials before the opening reads them
        msg0_grid = flock_combined_basis_msg_grid(n128, rs_lo);
        msg0_part = part_buf(*S, (size_t)msg0_grid * 3 * 16);
        FK(flock_launch_combined_basis_msg(n128, S->tlo0.p, S->thi0.p, S->tlo1.p, S->thi1.p, rs_lo, dt, dz, dbc,
                                           msg0_part, st));
      }
    }
    if (chain) {
      // packed-direct chain claim (pcs.rs:1055-1090): point [tau, sel0, 0^5, instance]
      tr.label("flock-pcs-packed-direct-v0");
      tr.observe(pd_value);
      F gpd = tr.sample();
      target += gpd * pd_value;
      const F et[2] = {F::one() + pd_tau, pd_tau}, es[2] = {F::one() + pd_sel0, pd_sel0};
      uint64_t c[8];
      for (int p = 0; p < 4; p++) u2(gpd * et[p & 1] * es[p >> 1], c + 2 * p);
      int lob = std::min(n_log, 12);
      eq_split_dev(*S, pd_inst, lob, S->eqlo, S->eqhi);
      FK(flock_launch_chain_claim_basis(dbc, (size_t)1 << n_log, S->eqlo.p, S->eqhi.p, lob, c, st));
    }
    T.ring_switch_ms = clk.lap();
    snap_waits(5);
    w.u64(2);
    w.fv(s_hat[0]);
    w.fv(s_hat[1]);

    // ---- Ligerito (ligerito.rs:6222-6980) ----
    tr.label("flock-ligerito-basis-v0");
    tr.observe(target);
    tr.observe_bytes(root0, 32);
    std::vector<std::pair<F, F>> msgs;
    std::vector<uint64_t> grind_nonces, fold_nonces;
    std::vector<F> ood_vals;
    void* dgr = S->grind.get(64);
    int grind_parity = 0;  // the grinds alternate two result slots, both cleared here once
    CK(cudaMemsetAsync(dgr, 0xFF, 16, st));
    auto grind = [&](uint32_t bits) {
      uint8_t dg[32];
      tr.digest(dg);
      uint64_t nonce = 0;
      uint64_t local_best = 0;
      uint64_t* h_best = S->pin ? reinterpret_cast<uint64_t*>(S->pin + kPinH2D) : &local_best;
      FK(flock_grind(dg, bits, dgr, &grind_parity, h_best, st, &S->waits, &nonce));
      tr.absorb_nonce(nonce);
      return nonce;
    };
    const int log_n = m - 7;
    // state: f in (fa_buf), b in (fb_buf), length len
    void* fcur = dz;  // the packed witness is consumed by the opening
    void* bcur = dbc;
    void* falt = S->f1.get(n128 / 2 * 16);
    void* balt = S->b1.get(n128 / 2 * 16);
    size_t len = n128;
    auto run_msg = [&](int fold, F rr) {
      size_t n_out = fold ? len / 2 : len;
      int grid = flock_lig_grid(n_out / 2);
      void* dpart = part_buf(*S, (size_t)grid * 3 * 16);
      uint64_t rp[2];
      u2(rr, rp);
      if (fold) {
        FK(flock_launch_lig_fold_msg(fcur, bcur, n_out, 1, rp, falt, balt, dpart, grid, st));
        std::swap(fcur, falt);
        std::swap(bcur, balt);
        len = n_out;
      } else {
        FK(flock_launch_lig_fold_msg(fcur, bcur, n_out, 0, rp, nullptr, nullptr, dpart, grid, st));
      }
      auto s = reduce_partials(*S, dpart, grid, 3);
      msgs.push_back({s[0], s[1]});
      tr.observe(s[0]);
      tr.observe(s[1]);
    };
    auto introduce = [&](const void* dbasis) {
      int grid = flock_lig_grid(len / 2);
      void* dpart = part_buf(*S, (size_t)grid * 3 * 16);
      uint64_t rp[2] = {0, 0};
      FK(flock_launch_lig_fold_msg(fcur, dbasis, len, 0, rp, nullptr, nullptr, dpart, grid, st));
      auto s = reduce_partials(*S, dpart, grid, 3);
      msgs.push_back({s[0], s[1]});
      tr.observe(s[0]);
      tr.observe(s[1]);
      F bt = tr.sample();
      uint64_t bp[2];
      u2(bt, bp);
      FK(flock_launch_glue(bcur, dbasis, len, bp, st));
    };
    auto ood = [&](int count) {
      for (int o = 0; o < count; o++) {
        int nv = ilog2(len);
        auto zp = tr.sample_vec(nv);
        int lob = std::min(nv, 12);
        eq_split_dev(*S, zp, lob, S->eqlo, S->eqhi);
        int grid = flock_lig_grid(len / 2);
        void* dpart = part_buf(*S, (size_t)grid * 3 * 16);
        FK(flock_launch_lig_intro_eq(fcur, len, S->eqlo.p, S->eqhi.p, lob, dpart, grid, st));
        auto s = reduce_partials(*S, dpart, grid, 3);
        tr.observe(s[2]);
        ood_vals.push_back(s[2]);
        msgs.push_back({s[0], s[1]});
        tr.observe(s[0]);
        tr.observe(s[1]);
        F bt = tr.sample();
        uint64_t bp[2];
        u2(bt, bp);
        FK(flock_launch_glue_eq(bcur, len, S->eqlo.p, S->eqhi.p, lob, bp, st));
      }
    };
    auto induce = [&](int nvars, const std::vector<uint32_t>& q, const std::vector<F>& alpha_v) {
      const Sks& sk = sks_for(nvars);
      auto aw = eq_table(alpha_v);
      aw.resize(q.size());
      // What_k(x^b) table of nvars: constant, copied to the device once
      if (nvars >= kSklMax) throw Fail(FLOCK_ERR_SHAPE, "basis table size");
      void* dsk = S->skl[nvars].p;
      if (!dsk) {
        dsk = S->skl[nvars].get((size_t)nvars * 32 * 16);
        h2d(*S, dsk, sk.lin.data(), (size_t)nvars * 32 * 16);
      }
      uint32_t* dq = (uint32_t*)S->qbuf.get(q.size() * 4);
      h2d(*S, dq, q.data(), q.size() * 4);
      void* dal = S->abuf.get(q.size() * 16);
      h2d(*S, dal, aw.data(), q.size() * 16);
      int lo_bits = flock_induce_basis_lo_bits(nvars), hi_bits = nvars - lo_bits;
      void* dW = S->W.get(q.size() * nvars * 16);
      void* dLO = S->LO.get((q.size() << lo_bits) * 16);
      void* dHI = S->HI.get((q.size() << hi_bits) * 16);
      void* dbs = S->basis.get(((size_t)16) << nvars);
      const size_t scr = flock_induce_basis_scratch_bytes(nvars);
      FK(flock_launch_induce_basis(dq, (int)q.size(), nvars, dsk, dal, dW, dLO, dHI, dbs,
                                   scr ? S->part.get(scr) : nullptr, st));
      return dbs;
    };

    if (msg0_grid) {  // computed with the combined basis
      auto s0 = reduce_partials(*S, msg0_part, msg0_grid, 3);
      msgs.push_back({s0[0], s0[1]});
      tr.observe(s0[0]);
      tr.observe(s0[1]);
    } else {
      run_msg(0, F());
    }
    for (int j = 0; j < cfg.initial_k; j++) {
      int bits = cfg.fold_bits[0] - j;
      if (bits > 0) fold_nonces.push_back(grind((uint32_t)bits));
      F rr = tr.sample();
      run_msg(1, rr);
    }
    int n1 = log_n - cfg.initial_k;
    int lni = cfg.ks[0];
    int cur_rate = cfg.rates[1];
    int slot = 0;
    uint8_t root_prev[32];
    std::vector<std::vector<uint8_t>> roots;
    void* pcw = S->lvl_cw[slot].get(((size_t)16 << (n1 + cur_rate)));
    void* ptree = S->lvl_tree[slot].get((2 * ((size_t)1 << (n1 - lni + cur_rate)) - 1) * 32);
    ligero_commit(*S, fcur, n1 - lni, lni, cur_rate, pcw, ptree, root_prev);
    roots.emplace_back(root_prev, root_prev + 32);
    tr.observe_bytes(root_prev, 32);
    size_t prev_block = (size_t)1 << (n1 - lni + cur_rate);
    int prev_width = 1 << lni;
    ood(cfg.ood[1]);
    grind_nonces.push_back(grind((uint32_t)cfg.grind_bits[0]));
    auto q0 = sample_queries(tr, block0, cfg.queries[0]);
    auto a0 = tr.sample_vec(ilog2(cfg.queries[0]));
    // the induced basis needs the queries only: its kernels are queued first
    // and run while the host prepares the opening (multiproof indices)
    void* dbs0 = induce(n1, q0, a0);
    Open open0 = open_rows(*S, dcw, dtree, block0, 1 << lbs, q0);
    introduce(dbs0);
    std::vector<Open> rec_opens;
    std::vector<F> yr;
    Open final_open;
    for (int i = 0; i < cfg.steps; i++) {
      int ki = cfg.ks[i];
      for (int j = 0; j < ki; j++) {
        int bits = cfg.fold_bits[i + 1] - j;
        if (bits > 0) fold_nonces.push_back(grind((uint32_t)bits));
        F rr = tr.sample();
        run_msg(1, rr);
      }
      if (i == cfg.steps - 1) {
        yr.resize(len);
        d2h(*S, yr.data(), fcur, len * 16);
        for (auto& v : yr) tr.observe(v);
        grind_nonces.push_back(grind((uint32_t)cfg.grind_bits[i + 1]));
        auto ql = sample_queries(tr, prev_block, cfg.queries[i + 1]);
        final_open = open_rows(*S, S->lvl_cw[slot].p, S->lvl_tree[slot].p, prev_block, prev_width, ql);
        break;
      }
      int n_next = ilog2(len);
      int lni2 = cfg.ks[i + 1];
      int rate2 = cfg.rates[i + 2];
      int ns = slot ^ 1;
      void* ncw = S->lvl_cw[ns].get(((size_t)16 << (n_next + rate2)));
      void* ntree = S->lvl_tree[ns].get((2 * ((size_t)1 << (n_next - lni2 + rate2)) - 1) * 32);
      uint8_t rootn[32];
      ligero_commit(*S, fcur, n_next - lni2, lni2, rate2, ncw, ntree, rootn);
      roots.emplace_back(rootn, rootn + 32);
      tr.observe_bytes(rootn, 32);
      ood(cfg.ood[i + 2]);
      grind_nonces.push_back(grind((uint32_t)cfg.grind_bits[i + 1]));
      auto qi = sample_queries(tr, prev_block, cfg.queries[i + 1]);
      auto ai = tr.sample_vec(ilog2(cfg.queries[i + 1]));
      void* dbs = induce(n_next, qi, ai);
      rec_opens.push_back(open_rows(*S, S->lvl_cw[slot].p, S->lvl_tree[slot].p, prev_block, prev_width, qi));
      introduce(dbs);
      slot = ns;
      prev_block = (size_t)1 << (n_next - lni2 + rate2);
      prev_width = 1 << lni2;
    }
    // one wait for the openings' queued copies (the final opening's gathers
    // are the last work of the phase)
    CK(flock_stream_wait(st, &S->waits));
    finish_open(*S, open0);
    for (Open& o : rec_opens) finish_open(*S, o);
    finish_open(*S, final_open);
    T.ligerito_ms = clk.lap();
    snap_waits(6);

    // ---- bundle tail: BatchOpeningProofLigerito.ligerito ----
    w.raw(root0, 32);  // initial_root
    write_open(w, open0);
    w.u64(roots.size());
    for (auto& rt : roots) w.raw(rt.data(), 32);
    w.u64(rec_opens.size());
    for (auto& o : rec_opens) write_open(w, o);
    w.fv(yr);
    write_open(w, final_open);
    w.pv(msgs);
    w.u64(grind_nonces.size());
    for (auto x : grind_nonces) w.u64(x);
    w.fv(ood_vals);
    w.u64(fold_nonces.size());
    for (auto x : fold_nonces) w.u64(x);
    if (chain) {
      // cv_0_phys, cv_last_phys: Vec<bool>, bit 32 w + b = bit b of word w (blake3.rs:3762-3770)
      for (const uint32_t* cv : {chain->cv0, chain->cv_last}) {
        w.u64(256);
        uint8_t bits[256];
        for (int i = 0; i < 256; i++) bits[i] = (uint8_t)((cv[i / 32] >> (i % 32)) & 1);
        w.raw(bits, 256);
      }
    }
    out.swap(w.v);
    if (ext_tr) *ext_tr = tr;
    if (S->timing) {
      for (int k = 0; k < kKernelSpans; k++) {
        S->span_ms[k] = 0;
        if (cudaEventSynchronize(S->tev[2 * k + 1]) == cudaSuccess)
          cudaEventElapsedTime(&S->span_ms[k], S->tev[2 * k], S->tev[2 * k + 1]);
      }
      cudaGetLastError();
    }
    T.serialize_ms = clk.lap();
    snap_waits(7);
    return FLOCK_OK;
  } catch (const Fail& f) {
    return f.code;
  } catch (const std::bad_alloc&) {
    return FLOCK_ERR_OOM;
  }
}

// ============================================================================
// Verifier (crates/flock-core/src/verifier.rs verify_ligerito, with
// R1csProofBundleLigerito::from_bytes, proof_io.rs:161-208): the transcript
// replay, the sumcheck checks, Merkle openings and proof-of-work checks run on
// the host; the parts that are linear in the witness size run on the device
// with the prover's kernels: the lincheck matrix fold A^T eq, B^T eq (lc_comb),
// the ring-switch combined basis (2^(m-7) positions) and its LSB folds down to
// the final Ligerito residual.
// ============================================================================
namespace {

struct Reader {
  const uint8_t* p;
  size_t n, off = 0;
  bool ok = true;
  bool take(void* dst, size_t k) {
    if (!ok || k > n - off) return ok = false;
    memcpy(dst, p + off, k);
    off += k;
    return true;
  }
  uint64_t u64() {
    uint64_t v = 0;
    take(&v, 8);
    return v;
  }
  uint32_t u32() {
    uint32_t v = 0;
    take(&v, 4);
    return v;
  }
  F f() {
    F v;
    v.lo = u64();
    v.hi = u64();
    return v;
  }
  // length-prefixed F128 vector with an upper bound on the length
  std::vector<F> fv(size_t max_len) {
    uint64_t k = u64();
    if (!ok || k > max_len || k * 16 > n - off) {
      ok = false;
      return {};
    }
    std::vector<F> v(k);
    take(v.data(), 16 * k);
    return v;
  }
  std::vector<std::pair<F, F>> pv(size_t max_len) {
    uint64_t k = u64();
    if (!ok || k > max_len || k * 32 > n - off) {
      ok = false;
      return {};
    }
    std::vector<std::pair<F, F>> v(k);
    for (auto& e : v) {
      e.first = f();
      e.second = f();
    }
    return v;
  }
  std::vector<uint64_t> u64v(size_t max_len) {
    uint64_t k = u64();
    if (!ok || k > max_len || k * 8 > n - off) {
      ok = false;
      return {};
    }
    std::vector<uint64_t> v(k);
    take(v.data(), 8 * k);
    return v;
  }
};

struct VOpen {
  std::vector<std::vector<F>> rows;
  std::vector<std::array<uint8_t, 32>> nodes;
};
bool read_open(Reader& r, VOpen& o) {
  uint64_t nq = r.u64();
  if (!r.ok || nq > (1u << 20)) return r.ok = false;
  o.rows.resize(nq);
  for (auto& row : o.rows) row = r.fv(1 << 12);
  uint64_t nn = r.u64();
  if (!r.ok || nn > (1u << 24) || nn * 32 > r.n - r.off) return r.ok = false;
  o.nodes.resize(nn);
  for (auto& h : o.nodes) r.take(h.data(), 32);
  return r.ok;
}

using H32 = std::array<uint8_t, 32>;
H32 cv_bytes(const uint32_t w[8]) {
  H32 h;
  memcpy(h.data(), w, 32);  // little-endian words
  return h;
}
// Non-root chaining value of a single-chunk leaf (<= 1024 bytes): blocks with
// counter 0, CHUNK_START on the first, CHUNK_END on the last (merkle.rs:200-210).
H32 leaf_cv(const uint8_t* d, size_t len) {
  uint32_t cv[8];
  memcpy(cv, hb3::IV, 32);
  size_t nb = len == 0 ? 1 : (len + 63) / 64;
  for (size_t b = 0; b < nb; b++) {
    size_t off = b * 64, bl = len - off < 64 ? len - off : 64;
    uint32_t m[16], o[16];
    hb3::load_words(d + off, bl, m);
    uint32_t fl = (b == 0 ? hb3::CHUNK_START : 0) | (b + 1 == nb ? hb3::CHUNK_END : 0);
    hb3::compress(cv, m, 0, (uint32_t)bl, fl, o);
    memcpy(cv, o, 32);
  }
  return cv_bytes(cv);
}
H32 parent_cv(const H32& l, const H32& r) {
  uint32_t m[16], o[16];
  memcpy(m, l.data(), 32);
  memcpy(m + 8, r.data(), 32);
  hb3::compress(hb3::IV, m, 0, 64, hb3::PARENT, o);
  return cv_bytes(o);
}
// Octopus multi-proof check (merkle.rs:937-1004).
bool merkle_multi_ok(const H32& root, size_t n_leaves, const std::vector<uint32_t>& pos, std::vector<H32> leaves,
                     const std::vector<H32>& proof) {
  if (n_leaves == 0 || (n_leaves & (n_leaves - 1)) || pos.size() != leaves.size()) return false;
  if (pos.empty()) return proof.empty();
  for (size_t i = 0; i < pos.size(); i++)
    if (pos[i] >= n_leaves || (i && pos[i - 1] >= pos[i])) return false;
  if (n_leaves == 1) return proof.empty() && leaves[0] == root;
  std::vector<std::pair<size_t, H32>> act;
  for (size_t i = 0; i < pos.size(); i++) act.push_back({pos[i], leaves[i]});
  size_t pi = 0;
  for (size_t ll = n_leaves; ll > 1; ll >>= 1) {
    std::vector<std::pair<size_t, H32>> nxt;
    for (size_t i = 0; i < act.size();) {
      size_t p = act[i].first;
      H32 l, r;
      if (i + 1 < act.size() && act[i + 1].first == (p ^ 1)) {
        l = act[i].second;
        r = act[i + 1].second;
        i += 2;
      } else {
        if (pi >= proof.size()) return false;
        const H32& sb = proof[pi++];
        if (p & 1) { l = sb; r = act[i].second; }
        else { l = act[i].second; r = sb; }
        i += 1;
      }
      nxt.push_back({p >> 1, parent_cv(l, r)});
    }
    act.swap(nxt);
  }
  return pi == proof.size() && act.size() == 1 && act[0].second == root;
}

// Proof of work (challenger.rs:1246-1310): BLAKE3(digest || nonce_le || 0^24)
// as one root block has >= bits leading zero bits, MSB first from byte 0.
bool pow_ok(fs::Transcript& tr, uint64_t nonce, uint32_t bits) {
  uint8_t dg[32];
  tr.digest(dg);
  uint8_t blk[64] = {0};
  memcpy(blk, dg, 32);
  memcpy(blk + 32, &nonce, 8);
  uint32_t m[16], o[16];
  hb3::load_words(blk, 64, m);
  hb3::compress(hb3::IV, m, 0, 64, hb3::CHUNK_START | hb3::CHUNK_END | hb3::ROOT, o);
  uint8_t h[32];
  memcpy(h, o, 32);
  uint32_t left = bits;
  for (int k = 0; k < 32 && left; k++) {
    if (left >= 8) {
      if (h[k]) return false;
      left -= 8;
    } else {
      if (h[k] >> (8 - left)) return false;
      left = 0;
    }
  }
  tr.absorb_nonce(nonce);
  return true;
}

struct Quad {
  F c, b, a;
  static Quad from(F u0, F u2, F t) { return {u0, t + u2, u2}; }
  F eval(F r) const { return c + r * b + r * r * a; }
  static Quad fold(const Quad& p, const Quad& q, F al) { return {p.c + al * q.c, p.b + al * q.b, p.a + al * q.a}; }
};

// Lagrange weights at z over all 128 nodes phi8(0..127), for the nodes
// 64..127 (multilinear.rs:522-548): the interpolant that vanishes on S.
std::vector<F> combined_weights(F z) {
  static const std::vector<F> den_inv = [] {
    std::vector<F> d(64);
    for (int i = 0; i < 64; i++) {
      F si = hf::phi8((uint8_t)(64 + i)), den = F::one();
      for (int j = 0; j < 128; j++)
        if (j != 64 + i) den = den * (si + hf::phi8((uint8_t)j));
      d[i] = hf::inv(den);
    }
    return d;
  }();
  std::vector<F> pre(129);
  pre[0] = F::one();
  for (int j = 0; j < 128; j++) pre[j + 1] = pre[j] * (z + hf::phi8((uint8_t)j));
  std::vector<F> w(64);
  F suf = F::one();
  std::vector<F> sufs(129);
  sufs[128] = F::one();
  for (int j = 127; j >= 0; j--) sufs[j] = sufs[j + 1] * (z + hf::phi8((uint8_t)j));
  for (int i = 0; i < 64; i++) w[i] = pre[64 + i] * sufs[65 + i] * den_inv[i];
  (void)suf;
  return w;
}

void bind_top(std::vector<F>& v, F r) {
  size_t half = v.size() / 2;
  for (size_t i = 0; i < half; i++) v[i] = v[i] + r * (v[i + half] + v[i]);
  v.resize(half);
}

std::vector<F> what_at(int n, const Sks& sk, uint32_t q) {
  std::vector<F> w(n);
  for (int k = 0; k < n; k++)
    for (int b = 0; b < 32; b++)
      if ((q >> b) & 1) w[k] += sk.lin[(size_t)k * 32 + b];
  return w;
}

// MLE of the induced basis at ris ++ bits(y) (ligerito.rs:1879-1987).
std::vector<F> induced_residual(int n, const std::vector<uint32_t>& q, const std::vector<F>& alpha, const F* ris,
                                int prefix, int yr_log) {
  const Sks& sk = sks_for(n);
  auto at = eq_table(alpha);
  std::vector<F> out((size_t)1 << yr_log);
  for (size_t i = 0; i < q.size(); i++) {
    auto w = what_at(n, sk, q[i]);
    F pre = F::one();
    for (int k = 0; k < prefix; k++) pre = pre * (F::one() + ris[k] * (F::one() + w[k]));
    F c = at[i] * pre;
    for (size_t y = 0; y < out.size(); y++) {
      F suf = c;
      for (int j = 0; j < yr_log; j++)
        if ((y >> j) & 1) suf = suf * w[prefix + j];
      out[y] += suf;
    }
  }
  return out;
}

// chain.rs:78-100: the successor relation's MLE.
F shift_mle(const std::vector<F>& a, const std::vector<F>& b) {
  const size_t n = a.size();
  std::vector<F> pre(n + 1, F::one()), suf(n + 1, F::one());
  for (size_t j = 0; j < n; j++) pre[j + 1] = pre[j] * (a[j] * (F::one() + b[j]));
  for (size_t j = n; j-- > 0;) suf[j] = suf[j + 1] * (F::one() + a[j] + b[j]);
  F acc;
  for (size_t j = 0; j < n; j++) acc += pre[j] * ((F::one() + a[j]) * b[j]) * suf[j + 1];
  return acc;
}

// chain_common.rs:88-113: the 256 endpoint bits packed into two words, eq(tau)-weighted.
F fold_phys(const std::vector<uint8_t>& bits, F tau) {
  F w[2];
  for (size_t i = 0; i < bits.size(); i++) {
    if (!bits[i]) continue;
    const size_t pos = i / 128, b = i % 128;
    if (b < 64) w[pos].lo ^= 1ULL << b;
    else w[pos].hi ^= 1ULL << (b - 64);
  }
  return (F::one() + tau) * w[0] + tau * w[1];
}

}  // namespace

// R1CS bundle (chain_domain == nullptr) or chain bundle under chain_domain.
static int verify_impl(ProverState* S, const uint8_t* data, size_t len, const char* chain_domain, int* accepted,
                std::string* why, fs::Transcript* ext_tr) {
  *accepted = 0;
  const bool chain = chain_domain != nullptr;
  auto reject = [&](const char* w) {
    if (why) *why = w;
    return FLOCK_OK;
  };
  try {
    CK(cudaSetDevice(S->device));
    CK(flock_stream_wait(S->st, &S->waits, false));
    S->pin_off = 0;
    cudaStream_t st = S->st;
    Reader rd{data, len};
    char magic[5];
    uint8_t ver[2];
    rd.take(magic, 5);
    rd.take(ver, 2);
    if (!rd.ok || memcmp(magic, "FLOCK", 5) != 0 || ver[0] != 4 || ver[1] != (chain ? 3 : 2)) return reject("header");
    if (chain && rd.u32() != 0) return reject("hash kind");  // HashKind::Blake3
    H32 root0;
    rd.take(root0.data(), 32);
    const uint64_t m64 = rd.u64(), rate0 = rd.u64(), lbs = rd.u64();
    const uint32_t profile = rd.u32(), hash_kind = rd.u32();
    if (!rd.ok || rate0 != 1 || lbs != 6 || profile != 0 || hash_kind != 1 || m64 < 22 || m64 > 35)
      return reject("params");
    const int m = (int)m64;
    LigCfg cfg;
    if (!lig_config(m, 0, cfg)) return reject("params");
    // zerocheck proof
    auto p_ab = rd.fv(64), p_c = rd.fv(64);
    auto zc_rounds = rd.pv(64);
    F fa = rd.f(), fb = rd.f(), final_c = rd.f();
    // lincheck proof
    auto lc_rounds = rd.pv(64);
    auto z_partial = rd.fv(64);
    // chain shift proof
    std::vector<std::pair<F, F>> sh_rounds;
    F sh_g;
    if (chain) {
      sh_rounds = rd.pv(64);
      sh_g = rd.f();
    }
    // ring switch
    uint64_t n_claims = rd.u64();
    auto sh0 = rd.fv(128), sh1 = rd.fv(128);
    // ligerito
    H32 init_root;
    rd.take(init_root.data(), 32);
    VOpen open0;
    read_open(rd, open0);
    std::vector<H32> roots(rd.u64());
    if (!rd.ok || roots.size() > 64) return reject("decode");
    for (auto& h : roots) rd.take(h.data(), 32);
    std::vector<VOpen> rec((size_t)rd.u64());
    if (!rd.ok || rec.size() > 64) return reject("decode");
    for (auto& o : rec) read_open(rd, o);
    auto yr = rd.fv((size_t)1 << 20);
    VOpen final_open;
    read_open(rd, final_open);
    auto msgs = rd.pv(1 << 12);
    auto grind_nonces = rd.u64v(64);
    auto ood_vals = rd.fv(64);
    auto fold_nonces = rd.u64v(1 << 10);
    std::vector<uint8_t> ends[2];
    if (chain)
      for (auto& e : ends) {
        const uint64_t k = rd.u64();
        if (!rd.ok || k > 256) return reject("chain endpoints");  // at most one 256-bit region
        e.resize(k);
        rd.take(e.data(), k);
        for (uint8_t x : e)
          if (x > 1) return reject("decode");
      }
    if (!rd.ok || rd.off != len) return reject("decode");
    if (p_ab.size() != 64 || p_c.size() != 64 || (int)zc_rounds.size() != m - 6 || lc_rounds.size() != 8 ||
        z_partial.size() != 64 || n_claims != 2 || sh0.size() != 128 || sh1.size() != 128)
      return reject("shape");

    uint8_t digest[32];
    flock_statement_digest(m, digest);
    fs::Transcript tr = ext_tr ? *ext_tr : fs::Transcript(chain ? chain_domain : "flock-bench-v0");
    tr.label("flock-r1cs-v0");
    tr.observe_bytes(digest, 32);
    tr.observe_bytes(root0.data(), 32);
    const Lagrange& LG = lagrange();

    // ---- zerocheck (zerocheck.rs:1365-1517) ----
    tr.label("flock-zerocheck-v0");
    std::vector<F> r(m);
    {
      auto rs = tr.sample_vec(6);
      auto ro = tr.sample_vec(m - 13);
      for (int i = 0; i < 6; i++) r[i] = rs[i];
      for (int i = 0; i < 3; i++) r[6 + i] = hf::phi8(zc::SMALL_CHAL[i]);
      for (int i = 0; i < 4; i++) {
        F g(1ULL << (1 << i), 0);
        r[9 + i] = g * hf::inv(F::one() + g);
      }
      for (int i = 13; i < m; i++) r[i] = ro[i - 13];
    }
    tr.observe_slice(p_ab.data(), 64);
    tr.observe_slice(p_c.data(), 64);
    const F z = tr.sample();
    {
      auto wl = LG.at(z, 1);
      if (dot(wl.data(), p_c.data(), 64) != final_c) return reject("zerocheck c-eval");
    }
    F running;
    {
      auto cw = combined_weights(z);
      auto wl = LG.at(z, 1);
      for (int i = 0; i < 64; i++) running += cw[i] * (p_ab[i] + p_c[i]) + wl[i] * p_c[i];
    }
    std::vector<F> rho;
    for (int i = 0; i < m - 6; i++) {
      F req = r[6 + i], g1 = zc_rounds[i].first, gi = zc_rounds[i].second;
      F g0 = (running + req * g1) * hf::inv(F::one() + req);
      tr.observe(g1);
      tr.observe(gi);
      F pch = tr.sample();
      rho.push_back(pch);
      F op = F::one() + pch;
      running = g0 * op + g1 * pch + gi * pch * op;
    }
    if (running != fa * fb) return reject("zerocheck sumcheck final");
    tr.observe(fa);
    tr.observe(fb);

    // ---- lincheck (lincheck.rs:1480-1660) ----
    const int inner_rest = 14 - 6;
    std::vector<F> x_in(rho.begin(), rho.begin() + inner_rest), x_out(rho.begin() + inner_rest, rho.end());
    tr.label("flock-lincheck-v0");
    F alpha = tr.sample();
    F beta = tr.sample();
    std::vector<F> comb(FLOCK_K);
    {
      if (!S->csc_ready) {
        const HostCsc& c = flock_host_csc();
        h2d(*S, S->csc_ap.get(c.a_ptr.size() * 4), c.a_ptr.data(), c.a_ptr.size() * 4);
        h2d(*S, S->csc_ai.get(c.a_idx.size() * 4), c.a_idx.data(), c.a_idx.size() * 4);
        h2d(*S, S->csc_bp.get(c.b_ptr.size() * 4), c.b_ptr.data(), c.b_ptr.size() * 4);
        h2d(*S, S->csc_bi.get(c.b_idx.size() * 4), c.b_idx.data(), c.b_idx.size() * 4);
        CK(flock_stream_wait(st, &S->waits, false));
        S->csc_ready = true;
      }
      auto lag_z = LG.at(z, 0);
      void* dlag = S->lag.get(64 * 16);
      h2d(*S, dlag, lag_z.data(), 64 * 16);
      void* dxr = S->small.get(inner_rest * 16);
      h2d(*S, dxr, x_in.data(), inner_rest * 16);
      void* deqin = S->eqin.get(FLOCK_K * 16);
      FK(flock_launch_lc_quirky_eq(dlag, dxr, inner_rest, deqin, st));
      void* dcomb = S->comb.get(FLOCK_K * 16);
      uint64_t al[2], be[2];
      u2(alpha, al);
      u2(beta, be);
      FK(flock_launch_lc_comb((const uint32_t*)S->csc_ap.p, (const uint32_t*)S->csc_ai.p, (const uint32_t*)S->csc_bp.p,
                              (const uint32_t*)S->csc_bi.p, deqin, al, be, 512, dcomb, st));
      d2h(*S, comb.data(), dcomb, FLOCK_K * 16);
    }
    running = alpha * fa + fb + beta;
    std::vector<F> rr;
    for (auto& rdm : lc_rounds) {
      tr.observe(rdm.first);
      tr.observe(rdm.second);
      F x = tr.sample();
      F e0 = running + rdm.first;
      F c1 = e0 + rdm.first + rdm.second;
      running = rdm.second * x * x + c1 * x + e0;
      bind_top(comb, x);
      rr.push_back(x);
    }
    tr.observe_slice(z_partial.data(), 64);
    if (dot(comb.data(), z_partial.data(), 64) != running) return reject("lincheck final");
    const F r_inner_skip = tr.sample();
    F lc_w;
    {
      auto l2 = LG.at(r_inner_skip, 0);
      lc_w = dot(l2.data(), z_partial.data(), 64);
    }
    std::vector<F> r_inner_rest(rr.rbegin(), rr.rend());

    // ---- chain: endpoints and shift sumcheck (chain_common.rs:366-377, chain.rs:238-302) ----
    std::vector<F> pd_inst;
    F pd_tau, pd_sel0;
    const int n_log = m - 14;
    if (chain) {
      pd_tau = tr.sample_vec(1)[0];
      const F x0 = fold_phys(ends[0], pd_tau), xl = fold_phys(ends[1], pd_tau);
      if ((int)sh_rounds.size() != n_log + 1) return reject("chain shift");
      auto tau = tr.sample_vec(n_log);
      const F al = tr.sample();
      F ones = F::one();
      for (auto& t : tau) ones = ones * t;
      F claim = ones * xl + al * x0;
      std::vector<F> rs;
      for (auto& q : sh_rounds) {
        tr.observe(q.first);
        tr.observe(q.second);
        F x = tr.sample();
        F e0 = claim + q.first;
        F c1 = e0 + q.first + q.second;
        claim = q.second * x * x + c1 * x + e0;
        rs.push_back(x);
      }
      pd_inst.assign(rs.rbegin(), rs.rend() - 1);
      pd_sel0 = rs[0];
      F eq_tt = F::one(), eq_t0 = F::one();
      for (int j = 0; j < n_log; j++) {
        eq_tt = eq_tt * (F::one() + tau[j] + pd_inst[j]);
        eq_t0 = eq_t0 * (F::one() + pd_inst[j]);
      }
      const F o0 = F::one() + pd_sel0;
      const F wfin = shift_mle(tau, pd_inst) * o0 + eq_tt * pd_sel0 + al * eq_t0 * o0;
      if (claim != wfin * sh_g) return reject("chain shift");
    }

    // ---- ring switch of [ab, c] (ring_switch.rs:2708-3345, pcs.rs:1025-1110) ----
    tr.label("flock-pcs-open-batch-v0");
    std::vector<F> x_ab(r_inner_rest);
    x_ab.insert(x_ab.end(), x_out.begin(), x_out.end());
    std::vector<F> x_c(r.begin() + 6, r.end());
    const std::vector<F>* xs[2] = {&x_ab, &x_c};
    const std::vector<F>* shs[2] = {&sh0, &sh1};
    const F zsk[2] = {r_inner_skip, z}, val[2] = {lc_w, final_c};
    DBuf* tlo[2] = {&S->tlo0, &S->tlo1};
    DBuf* thi[2] = {&S->thi0, &S->thi1};
    std::vector<F> eqr[2];
    F claims[2];
    const int L = m - 7;
    const int rs_lo = std::min(13, L - 1);
    for (int k = 0; k < 2; k++) {
      tr.label("flock-ring-switch-v0");
      tr.observe_slice(shs[k]->data(), 128);
      auto Ls = LG.at(zsk[k], 0);
      F x0 = (*xs[k])[0], acc;
      for (int i = 0; i < 128; i++) acc += Ls[i & 63] * ((i >> 6) & 1 ? x0 : F::one() + x0) * (*shs[k])[i];
      if (acc != val[k]) return reject("ring switch claim");
      auto rpp = tr.sample_vec(7);
      eqr[k] = eq_table(rpp);
      auto u = transpose128(*shs[k]);
      claims[k] = dot(u.data(), eqr[k].data(), 128);
      std::vector<F> suffix(xs[k]->begin() + 1, xs[k]->end());
      eq_split_dev(*S, suffix, rs_lo, *tlo[k], *thi[k]);
    }
    F gam[2] = {tr.sample(), tr.sample()};
    F target = gam[0] * claims[0] + gam[1] * claims[1];
    const size_t n128 = (size_t)1 << L;
    void* dbc = S->bc.get(n128 * 16);
    {
      std::vector<F> wk(2 * 128);
      for (int k = 0; k < 2; k++)
        for (int bb = 0; bb < 128; bb++) wk[k * 128 + bb] = gam[k] * eqr[k][bb];
      void* dt = S->tables.get(wk.size() * 16);
      h2d(*S, dt, wk.data(), wk.size() * 16);
      FK(flock_launch_combined_basis(n128, S->tlo0.p, S->thi0.p, S->tlo1.p, S->thi1.p, rs_lo, dt, dbc, st));
    }
    if (chain) {
      // packed-direct chain claim (pcs.rs:1755-1770): its eq tensor joins the basis
      tr.label("flock-pcs-packed-direct-v0");
      tr.observe(sh_g);
      F gpd = tr.sample();
      target += gpd * sh_g;
      const F et[2] = {F::one() + pd_tau, pd_tau}, es[2] = {F::one() + pd_sel0, pd_sel0};
      uint64_t c[8];
      for (int p = 0; p < 4; p++) u2(gpd * et[p & 1] * es[p >> 1], c + 2 * p);
      int lob = std::min(n_log, 12);
      eq_split_dev(*S, pd_inst, lob, S->eqlo, S->eqhi);
      FK(flock_launch_chain_claim_basis(dbc, (size_t)1 << n_log, S->eqlo.p, S->eqhi.p, lob, c, st));
    }

    // ---- Ligerito (ligerito.rs:6981-8544) ----
    if (init_root != root0) return reject("ligerito root");
    tr.label("flock-ligerito-basis-v0");
    tr.observe(target);
    tr.observe_bytes(root0.data(), 32);
    const int log_n = L, k0 = cfg.initial_k, R = cfg.steps;
    const size_t block0 = (size_t)1 << (log_n - k0 + cfg.rates[0]);
    F t_r = target;
    size_t tx = 0, fni = 0, oi = 0, ni = 0, rp = 0;
    std::pair<F, F> msg;
    auto next_msg = [&]() {
      if (tx >= msgs.size()) return false;
      msg = msgs[tx++];
      tr.observe(msg.first);
      tr.observe(msg.second);
      return true;
    };
    auto fold_pow = [&](int lvl, int j) -> bool {
      int bits = cfg.fold_bits[lvl] - j;
      if (bits <= 0) return true;
      return fni < fold_nonces.size() && pow_ok(tr, fold_nonces[fni++], (uint32_t)bits);
    };
    auto opens_ok = [&](const H32& root, size_t block_len, const std::vector<uint32_t>& q, const VOpen& o,
                        size_t width) {
      if (q.size() != o.rows.size()) return false;
      std::vector<H32> leaves;
      for (auto& row : o.rows) {
        if (row.size() != width) return false;
        leaves.push_back(leaf_cv((const uint8_t*)row.data(), row.size() * 16));
      }
      std::vector<H32> nodes(o.nodes.begin(), o.nodes.end());
      return merkle_multi_ok(root, block_len, q, leaves, nodes);
    };
    auto enforced = [&](const VOpen& o, const std::vector<F>& v, const std::vector<F>& a) {
      auto eqv = eq_table(v);
      auto at = eq_table(a);
      F sum;
      for (size_t i = 0; i < o.rows.size(); i++) sum += at[i] * dot(o.rows[i].data(), eqv.data(), o.rows[i].size());
      return sum;
    };
    struct OodCtx { std::vector<F> z; size_t start; F beta; };
    struct LvlCtx { int n; std::vector<uint32_t> q; std::vector<F> alpha; size_t start; F beta; };
    std::vector<OodCtx> oods;
    std::vector<LvlCtx> lvls;
    std::vector<F> ris;
    if (!next_msg()) return reject("ligerito transcript");
    Quad run = Quad::from(msg.first, msg.second, t_r);
    for (int j = 0; j < k0; j++) {
      if (!fold_pow(0, j)) return reject("ligerito fold pow");
      F x = tr.sample();
      ris.push_back(x);
      t_r = run.eval(x);
      if (!next_msg()) return reject("ligerito transcript");
      run = Quad::from(msg.first, msg.second, t_r);
    }
    if (roots.empty()) return reject("ligerito roots");
    H32 prev_root = roots[0];
    tr.observe_bytes(prev_root.data(), 32);
    const int n1 = log_n - k0;
    auto do_ood = [&](int count, int nv, size_t start) -> bool {
      for (int o = 0; o < count; o++) {
        auto zp = tr.sample_vec(nv);
        if (oi >= ood_vals.size()) return false;
        F y = ood_vals[oi++];
        tr.observe(y);
        if (!next_msg()) return false;
        Quad iq = Quad::from(msg.first, msg.second, y);
        F bt = tr.sample();
        run = Quad::fold(run, iq, bt);
        t_r += bt * y;
        oods.push_back({zp, start, bt});
      }
      return true;
    };
    if (!do_ood(cfg.ood[1], n1, (size_t)k0)) return reject("ligerito ood");
    if (ni >= grind_nonces.size() || !pow_ok(tr, grind_nonces[ni++], (uint32_t)cfg.grind_bits[0]))
      return reject("ligerito query pow");
    auto q0 = sample_queries(tr, block0, cfg.queries[0]);
    auto a0 = tr.sample_vec(ilog2(cfg.queries[0]));
    if (!opens_ok(init_root, block0, q0, open0, (size_t)1 << k0)) return reject("ligerito L0 opens");
    {
      F es0 = enforced(open0, ris, a0);
      if (!next_msg()) return reject("ligerito transcript");
      Quad iq = Quad::from(msg.first, msg.second, es0);
      F bt = tr.sample();
      run = Quad::fold(run, iq, bt);
      t_r += bt * es0;
      lvls.push_back({n1, q0, a0, (size_t)k0, bt});
    }
    int prev_lni = cfg.ks[0], prev_lmc = n1 - prev_lni, prev_rate = cfg.rates[1];
    int n_cur = n1;
    for (int i = 0; i < R; i++) {
      const int ki = cfg.ks[i];
      std::vector<F> level_rs;
      for (int j = 0; j < ki; j++) {
        if (!fold_pow(i + 1, j)) return reject("ligerito fold pow");
        F x = tr.sample();
        ris.push_back(x);
        level_rs.push_back(x);
        t_r = run.eval(x);
        if (!next_msg()) return reject("ligerito transcript");
        run = Quad::from(msg.first, msg.second, t_r);
      }
      n_cur -= ki;
      const size_t pbl = (size_t)1 << (prev_lmc + prev_rate);
      if (i == R - 1) {
        if (tx != msgs.size() || oi != ood_vals.size() || fni != fold_nonces.size()) return reject("ligerito trailing");
        if (yr.size() != ((size_t)1 << n_cur)) return reject("ligerito yr size");
        for (auto& v : yr) tr.observe(v);
        if (ni >= grind_nonces.size() || !pow_ok(tr, grind_nonces[ni], (uint32_t)cfg.grind_bits[i + 1]))
          return reject("ligerito last query pow");
        auto ql = sample_queries(tr, pbl, cfg.queries[i + 1]);
        auto alv = tr.sample_vec(ilog2(cfg.queries[i + 1]));
        if (!opens_ok(prev_root, pbl, ql, final_open, (size_t)1 << prev_lni)) return reject("ligerito last opens");
        F esl = enforced(final_open, level_rs, alv);
        F bl = tr.sample();
        t_r += bl * esl;
        lvls.push_back({n_cur, ql, alv, ris.size(), bl});
        const int yl = n_cur;
        // dense residual of the combined basis: LSB folds at every r on the device
        std::vector<F> bres((size_t)1 << yl);
        {
          void* cur = dbc;
          void* alt = S->f1.get(n128 / 2 * 16);
          void* alt2 = S->b1.get(n128 / 2 * 16);
          size_t nlen = n128;
          if (((size_t)1 << (yl + ris.size())) != n128) return reject("ligerito residual size");
          for (size_t t = 0; t < ris.size(); t++) {
            uint64_t rp2[2];
            u2(ris[t], rp2);
            void* dst = (cur == alt) ? alt2 : alt;
            FK(flock_launch_fold_lsb(cur, nlen / 2, rp2, dst, st));
            cur = dst;
            nlen /= 2;
          }
          d2h(*S, bres.data(), cur, bres.size() * 16);
        }
        std::vector<F> cy(bres);
        for (auto& c : lvls) {
          auto ind = induced_residual(c.n, c.q, c.alpha, ris.data() + c.start, c.n - yl, yl);
          for (size_t y = 0; y < cy.size(); y++) cy[y] += c.beta * ind[y];
        }
        for (auto& c : oods) {
          int folded = (int)c.z.size() - yl;
          F sc = c.beta;
          for (int b2 = 0; b2 < folded; b2++) sc = sc * (F::one() + c.z[b2] + ris[c.start + b2]);
          std::vector<F> tail(c.z.begin() + folded, c.z.end());
          auto t = eq_table(tail);
          for (size_t y = 0; y < cy.size(); y++) cy[y] += sc * t[y];
        }
        F inner = dot(yr.data(), cy.data(), cy.size());
        if (inner != t_r) return reject("ligerito residual check");
        *accepted = 1;
        if (ext_tr) *ext_tr = tr;
        if (why) *why = "ok";
        return FLOCK_OK;
      }
      if ((size_t)(i + 1) >= roots.size()) return reject("ligerito roots");
      H32 root_next = roots[i + 1];
      tr.observe_bytes(root_next.data(), 32);
      if (!do_ood(cfg.ood[i + 2], n_cur, ris.size())) return reject("ligerito ood");
      if (ni >= grind_nonces.size() || !pow_ok(tr, grind_nonces[ni++], (uint32_t)cfg.grind_bits[i + 1]))
        return reject("ligerito query pow");
      auto qi = sample_queries(tr, pbl, cfg.queries[i + 1]);
      auto ai = tr.sample_vec(ilog2(cfg.queries[i + 1]));
      if (rp >= rec.size()) return reject("ligerito openings");
      const VOpen& lo = rec[rp++];
      if (!opens_ok(prev_root, pbl, qi, lo, (size_t)1 << prev_lni)) return reject("ligerito level opens");
      F esi = enforced(lo, level_rs, ai);
      if (!next_msg()) return reject("ligerito transcript");
      Quad iq = Quad::from(msg.first, msg.second, esi);
      F bt = tr.sample();
      run = Quad::fold(run, iq, bt);
      t_r += bt * esi;
      lvls.push_back({n_cur, qi, ai, ris.size(), bt});
      prev_root = root_next;
      prev_lni = cfg.ks[i + 1];
      prev_lmc = n_cur - prev_lni;
      prev_rate = cfg.rates[i + 2];
    }
    return reject("ligerito steps");
  } catch (const Fail& f) {
    return f.code;
  }
}

int flock_prover_verify(ProverState* S, const uint8_t* data, size_t len, int* accepted, std::string* why,
                        fs::Transcript* tr) {
  return verify_impl(S, data, len, nullptr, accepted, why, tr);
}

int flock_prover_verify_chain(ProverState* S, const uint8_t* data, size_t len, const char* domain, int* accepted,
                              std::string* why) {
  return verify_impl(S, data, len, domain ? domain : "flock_chain-cli", accepted, why, nullptr);
}
