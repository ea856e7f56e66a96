// Setup-time R1CS data for the BLAKE3 circuit: base matrices A_0, B_0, the
// statement digest and a column-major copy of the matrices for the lincheck
// comb gather.
//
// The rows restate build_matrices (crates/flock-prover/src/r1cs_hashes/blake3.rs:485-631):
// every bit of a symbolic 32-bit word is a GF(2) combination of witness
// slots, kept sorted and square-free (r1cs_hashes/common.rs:767-783); ADD
// x + y writes 31 carry rows a = x_i + carries_<i, b = y_i + carries_<i and
// yields sum_i = x_i + y_i + carries_<i. The digest is BLAKE3 over
// "flock-r1cs-stmt-v1" || m || k_log || k_skip || layout || A || B || C with
// length-prefixed little-endian u64 rows (crates/flock-core/src/r1cs.rs:343-460).
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "host_blake3.h"
#include "r1cs_setup.h"

namespace {

using Lin = std::vector<uint32_t>;
constexpr int K = 1 << 14;
constexpr int CONST_POS = 512, M_BASE = 513, T_LO = 1025, T_HI = 1057, BLEN = 1089, FLAGS = 1121, GS = 1153,
              GSTRIDE = 250, OUT_LO = 256, OUT_HI = 15153;
constexpr int LANES[8][4] = {{0, 4, 8, 12}, {1, 5, 9, 13}, {2, 6, 10, 14}, {3, 7, 11, 15},
                             {0, 5, 10, 15}, {1, 6, 11, 12}, {2, 7, 8, 13}, {3, 4, 9, 14}};
constexpr int PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
constexpr uint32_t IV4[4] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a};

Lin sym_xor(const Lin& x, const Lin& y) {
  Lin o;
  o.reserve(x.size() + y.size());
  std::set_symmetric_difference(x.begin(), x.end(), y.begin(), y.end(), std::back_inserter(o));
  return o;
}
struct Word {
  Lin b[32];
};
Word slots(int base) {
  Word w;
  for (int i = 0; i < 32; i++) w.b[i] = {(uint32_t)(base + i)};
  return w;
}
Word constant(uint32_t v) {
  Word w;
  for (int i = 0; i < 32; i++)
    if ((v >> i) & 1) w.b[i] = {(uint32_t)CONST_POS};
  return w;
}
Word wxor(const Word& x, const Word& y) {
  Word w;
  for (int i = 0; i < 32; i++) w.b[i] = sym_xor(x.b[i], y.b[i]);
  return w;
}
Word wrot(const Word& x, int n) {
  Word w;
  for (int i = 0; i < 32; i++) w.b[i] = x.b[(i + n) & 31];
  return w;
}

struct Mats {
  std::vector<Lin> A, B;
};

Word add(Mats& M, const Word& x, const Word& y, int base) {
  Lin carries;
  Word s;
  for (int i = 0; i < 32; i++) {
    if (i < 31) {
      M.A[base + i] = sym_xor(x.b[i], carries);
      M.B[base + i] = sym_xor(y.b[i], carries);
    }
    s.b[i] = sym_xor(sym_xor(x.b[i], y.b[i]), carries);
    if (i < 31) carries.push_back((uint32_t)(base + i));
  }
  return s;
}

void lin_rows(Mats& M, int base, const Word& w) {
  for (int i = 0; i < 32; i++) {
    M.A[base + i] = w.b[i];
    M.B[base + i] = {(uint32_t)CONST_POS};
  }
}

Mats build() {
  Mats M;
  M.A.assign(K, {});
  M.B.assign(K, {});
  M.A[CONST_POS] = {(uint32_t)CONST_POS};
  M.B[CONST_POS] = {(uint32_t)CONST_POS};
  auto input = [&](int base, int n) {
    for (int j = 0; j < n; j++) {
      M.A[base + j] = {(uint32_t)(base + j)};
      M.B[base + j] = {(uint32_t)CONST_POS};
    }
  };
  input(0, 256);
  input(M_BASE, 512);
  input(T_LO, 32);
  input(T_HI, 32);
  input(BLEN, 32);
  input(FLAGS, 32);
  Word st[16];
  for (int w = 0; w < 8; w++) st[w] = slots(32 * w);
  for (int i = 0; i < 4; i++) st[8 + i] = constant(IV4[i]);
  st[12] = slots(T_LO);
  st[13] = slots(T_HI);
  st[14] = slots(BLEN);
  st[15] = slots(FLAGS);
  int perm[16];
  for (int i = 0; i < 16; i++) perm[i] = i;
  for (int r = 0; r < 7; r++) {
    for (int gi = 0; gi < 8; gi++) {
      int g = 8 * r + gi, cb = GS + GSTRIDE * g, lb = cb + 186;
      const int* L = LANES[gi];
      Word a = st[L[0]], b = st[L[1]], c = st[L[2]], d = st[L[3]];
      Word mx = slots(M_BASE + 32 * perm[2 * gi]), my = slots(M_BASE + 32 * perm[2 * gi + 1]);
      Word t0 = add(M, a, b, cb);
      Word a1 = add(M, t0, mx, cb + 31);
      Word d1 = wrot(wxor(d, a1), 16);
      Word c1 = add(M, c, d1, cb + 62);
      Word b1 = wrot(wxor(b, c1), 12);
      Word t1 = add(M, a1, b1, cb + 93);
      Word a2 = add(M, t1, my, cb + 124);
      Word d2 = wrot(wxor(d1, a2), 8);
      Word c2 = add(M, c1, d2, cb + 155);
      Word bn = wrot(wxor(b1, c2), 7);
      lin_rows(M, lb, bn);
      lin_rows(M, lb + 32, d2);
      st[L[0]] = a2;
      st[L[1]] = slots(lb);
      st[L[2]] = c2;
      st[L[3]] = slots(lb + 32);
    }
    int next[16];
    for (int i = 0; i < 16; i++) next[i] = perm[PERM[i]];
    memcpy(perm, next, sizeof(perm));
  }
  for (int w = 0; w < 8; w++) {
    lin_rows(M, OUT_LO + 32 * w, wxor(st[w], st[w + 8]));
    lin_rows(M, OUT_HI + 32 * w, wxor(st[w + 8], slots(32 * w)));
  }
  return M;
}

void absorb_u64(hb3::Hasher& h, uint64_t v) { h.update(&v, 8); }
void absorb_rows(hb3::Hasher& h, const std::vector<Lin>& rows) {
  absorb_u64(h, K);
  absorb_u64(h, K);
  std::vector<uint64_t> buf;
  for (const auto& r : rows) {
    buf.assign(1, r.size());
    for (uint32_t c : r) buf.push_back(c);
    h.update(buf.data(), buf.size() * 8);
  }
}

void to_csc(const std::vector<Lin>& rows, std::vector<uint32_t>& ptr, std::vector<uint32_t>& idx) {
  ptr.assign(K + 1, 0);
  for (const auto& r : rows)
    for (uint32_t c : r) ptr[c + 1]++;
  for (int c = 0; c < K; c++) ptr[c + 1] += ptr[c];
  idx.assign(ptr[K], 0);
  std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int r = 0; r < K; r++)
    for (uint32_t c : rows[r]) idx[fill[c]++] = (uint32_t)r;
}

std::mutex g_mu;
Mats* g_mats = nullptr;
std::map<int, std::vector<uint8_t>> g_digests;
HostCsc* g_csc = nullptr;

const Mats& mats() {
  if (!g_mats) g_mats = new Mats(build());
  return *g_mats;
}

}  // namespace

void flock_statement_digest(int m, uint8_t out[32]) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_digests.find(m);
  if (it == g_digests.end()) {
    const Mats& M = mats();
    hb3::Hasher h;
    const char* label = "flock-r1cs-stmt-v1";
    h.update(label, strlen(label));
    absorb_u64(h, (uint64_t)m);
    absorb_u64(h, 14);
    absorb_u64(h, 6);
    uint8_t layout = 0;  // row-major
    h.update(&layout, 1);
    absorb_rows(h, M.A);
    absorb_rows(h, M.B);
    std::vector<Lin> C(K);
    for (int i = 0; i < K; i++) C[i] = {(uint32_t)i};
    absorb_rows(h, C);
    std::vector<uint8_t> d(32);
    h.finalize(d.data());
    it = g_digests.emplace(m, d).first;
  }
  memcpy(out, it->second.data(), 32);
}

const HostCsc& flock_host_csc() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_csc) {
    const Mats& M = mats();
    g_csc = new HostCsc;
    to_csc(M.A, g_csc->a_ptr, g_csc->a_idx);
    to_csc(M.B, g_csc->b_ptr, g_csc->b_idx);
  }
  return *g_csc;
}
