// Inputs, BLAKE3 R1CS witness, base matrices and statement digest for the
// oracle (test infrastructure only).
#include <algorithm>
#include <cstring>

#include "oracle.h"

namespace oracle {

// ---------------------------------------------------------------------------
// Input generator: benchmark-tools/common/src/lib.rs:4-33. SplitMix64 stream
// seeded with seed ^ rotl(log2, 29); each draw keeps the low 32 bits; the
// counter is a single u32 draw (high word zero); block_len 64, flags 11.
// ---------------------------------------------------------------------------
struct SplitMix {
  uint64_t s;
  uint32_t next_u32() {
    s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return (uint32_t)(z ^ (z >> 31));
  }
};

static std::vector<Compression> draw(uint64_t state, size_t count) {
  SplitMix rng{state};
  std::vector<Compression> out(count);
  for (auto& c : out) {
    for (int i = 0; i < 8; i++) c.cv[i] = rng.next_u32();
    for (int i = 0; i < 16; i++) c.m[i] = rng.next_u32();
    c.counter = rng.next_u32();
    c.block_len = 64;
    c.flags = 11;
  }
  return out;
}

std::vector<Compression> generate_compressions(uint32_t log2_size, uint64_t seed) {
  uint64_t l = log2_size;
  uint64_t rot = (l << 29) | (l >> 35);
  return draw(seed ^ rot, (size_t)1 << log2_size);
}

std::vector<Compression> canary_compressions(uint32_t log2_size) {
  size_t n = (size_t)1 << log2_size;
  return draw(0xC0FFEEBEEFULL ^ (uint64_t)n, n);
}

int min_n_blocks_log(size_t n) {
  if (n < 8) n = 8;
  int l = 0;
  while (((size_t)1 << l) < n) l++;
  return l;
}

// ---------------------------------------------------------------------------
// Witness layout, crates/flock-prover/src/r1cs_hashes/blake3.rs:107-231.
// ---------------------------------------------------------------------------
static constexpr int CV_BASE = 0, OUT_LO_BASE = 256, M_BASE = 513, T_LO_BASE = 1025,
                     T_HI_BASE = 1057, BLEN_BASE = 1089, FLAGS_BASE = 1121, GS_BASE = 1153,
                     G_STRIDE = 250, OUT_HI_BASE = 15153;
static const int G_LANES[8][4] = {{0, 4, 8, 12}, {1, 5, 9, 13}, {2, 6, 10, 14}, {3, 7, 11, 15},
                                  {0, 5, 10, 15}, {1, 6, 11, 12}, {2, 7, 8, 13}, {3, 4, 9, 14}};
static const int PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

// Per round r and G index g, the two message word indices (blake3.rs:313-345).
static void msg_schedule(int idx[7][8][2]) {
  int perm[16];
  for (int i = 0; i < 16; i++) perm[i] = i;
  for (int r = 0; r < 7; r++) {
    for (int g = 0; g < 8; g++) {
      idx[r][g][0] = perm[2 * g];
      idx[r][g][1] = perm[2 * g + 1];
    }
    int next[16];
    for (int i = 0; i < 16; i++) next[i] = perm[PERM[i]];
    memcpy(perm, next, sizeof(perm));
  }
}

static inline int carry_base(int g, int add_idx) { return GS_BASE + G_STRIDE * g + 31 * add_idx; }
static inline int lin_base(int g, int which) { return GS_BASE + G_STRIDE * g + 186 + 32 * which; }
static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

struct BlockBits {
  uint64_t z[K / 64], a[K / 64], b[K / 64];
  void put(uint64_t* v, int pos, uint32_t val, int width) {
    uint64_t x = width == 32 ? val : (val & ((1u << width) - 1));
    v[pos >> 6] |= x << (pos & 63);
    if ((pos & 63) + width > 64) v[(pos >> 6) + 1] |= x >> (64 - (pos & 63));
  }
  // Input / lin-id slot: z = a = value, b = all ones (blake3.rs:1150-1160).
  void lin(int pos, uint32_t val) { put(z, pos, val, 32); put(a, pos, val, 32); put(b, pos, 0xFFFFFFFFu, 32); }
  // Carry-only ADD (r1cs_hashes/common.rs:85-101): z = carry_aux, a = x^cin,
  // b = y^cin on bits 0..30.
  uint32_t add(uint32_t x, uint32_t y, int base) {
    uint32_t sum = x + y;
    uint32_t cin = sum ^ x ^ y;
    uint32_t left = (x ^ cin) & 0x7FFFFFFFu, right = (y ^ cin) & 0x7FFFFFFFu;
    put(z, base, left & right, 31);
    put(a, base, left, 31);
    put(b, base, right, 31);
    return sum;
  }
};

// One compression's witness rows; blake3.rs:965-1076 semantics.
static const int (*schedule())[8][2] {
  static int sched[7][8][2];
  static bool init = (msg_schedule(sched), true);
  (void)init;
  return sched;
}

static void build_block(const Compression& c, BlockBits& w) {
  const int (*sched)[8][2] = schedule();
  memset(&w, 0, sizeof(w));
  w.put(w.z, Z_CONST_POS, 1, 1);
  w.put(w.a, Z_CONST_POS, 1, 1);
  w.put(w.b, Z_CONST_POS, 1, 1);
  for (int i = 0; i < 8; i++) w.lin(CV_BASE + 32 * i, c.cv[i]);
  for (int i = 0; i < 16; i++) w.lin(M_BASE + 32 * i, c.m[i]);
  uint32_t t_lo = (uint32_t)c.counter, t_hi = (uint32_t)(c.counter >> 32);
  w.lin(T_LO_BASE, t_lo);
  w.lin(T_HI_BASE, t_hi);
  w.lin(BLEN_BASE, c.block_len);
  w.lin(FLAGS_BASE, c.flags);
  uint32_t s[16] = {c.cv[0], c.cv[1], c.cv[2], c.cv[3], c.cv[4], c.cv[5], c.cv[6], c.cv[7],
                    B3_IV[0], B3_IV[1], B3_IV[2], B3_IV[3], t_lo, t_hi, c.block_len, c.flags};
  for (int r = 0; r < 7; r++) {
    for (int gi = 0; gi < 8; gi++) {
      int g = r * 8 + gi;
      const int* L = G_LANES[gi];
      uint32_t mx = c.m[sched[r][gi][0]], my = c.m[sched[r][gi][1]];
      uint32_t a = s[L[0]], b = s[L[1]], cc = s[L[2]], d = s[L[3]];
      uint32_t tmp0 = w.add(a, b, carry_base(g, 0));
      uint32_t a1 = w.add(tmp0, mx, carry_base(g, 1));
      uint32_t d1 = rotr(d ^ a1, 16);
      uint32_t c1 = w.add(cc, d1, carry_base(g, 2));
      uint32_t b1 = rotr(b ^ c1, 12);
      uint32_t tmp1 = w.add(a1, b1, carry_base(g, 3));
      uint32_t a2 = w.add(tmp1, my, carry_base(g, 4));
      uint32_t d2 = rotr(d1 ^ a2, 8);
      uint32_t c2 = w.add(c1, d2, carry_base(g, 5));
      uint32_t b_new = rotr(b1 ^ c2, 7);
      w.lin(lin_base(g, 0), b_new);
      w.lin(lin_base(g, 1), d2);
      s[L[0]] = a2;
      s[L[1]] = b_new;
      s[L[2]] = c2;
      s[L[3]] = d2;
    }
  }
  for (int i = 0; i < 8; i++) {
    w.lin(OUT_LO_BASE + 32 * i, s[i] ^ s[i + 8]);
    w.lin(OUT_HI_BASE + 32 * i, s[i + 8] ^ c.cv[i]);
  }
}

Witness build_witness(const std::vector<Compression>& blocks, int n_blocks_log, bool with_stripe) {
  Witness out;
  out.m = K_LOG + n_blocks_log;
  size_t n_total = (size_t)1 << n_blocks_log;
  size_t per = K / 128;
  out.z.resize(n_total * per);
  out.a.resize(n_total * per);
  out.b.resize(n_total * per);
  Compression pad;
  memset(&pad, 0, sizeof(pad));
#pragma omp parallel for schedule(static)
  for (int64_t jj = 0; jj < (int64_t)n_total; jj++) {
    size_t j = (size_t)jj;
    BlockBits w;
    const Compression& c = j < blocks.size() ? blocks[j] : pad;
    build_block(c, w);
    for (size_t i = 0; i < per; i++) {
      out.z[j * per + i] = f128(w.z[2 * i], w.z[2 * i + 1]);
      out.a[j * per + i] = f128(w.a[2 * i], w.a[2 * i + 1]);
      out.b[j * per + i] = f128(w.b[2 * i], w.b[2 * i + 1]);
    }
  }
  if (with_stripe) {
    // Byte (byte_idx*K + i_inner), bit r = bit i_inner of compression
    // 8*byte_idx + r (crates/flock-core/src/lincheck.rs:88-110).
    out.stripe.assign(n_total * K / 8, 0);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)(n_total / 8); g++)
    for (size_t j = (size_t)g * 8; j < (size_t)g * 8 + 8; j++) {
      const uint64_t* zb = (const uint64_t*)&out.z[j * per];
      size_t byte_idx = j >> 3;
      int r = (int)(j & 7);
      for (int i = 0; i < K; i++)
        if ((zb[i >> 6] >> (i & 63)) & 1) out.stripe[byte_idx * K + i] |= (uint8_t)(1u << r);
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Base matrices, blake3.rs:485-631. A symbolic word bit is a GF(2) linear
// combination of slots kept as a sorted, square-free index list, which is the
// canonical row form of r1cs_hashes/common.rs:767-783.
// ---------------------------------------------------------------------------
using Lin = std::vector<uint32_t>;
static Lin lin_xor(const Lin& x, const Lin& y) {
  Lin out;
  out.reserve(x.size() + y.size());
  size_t i = 0, j = 0;
  while (i < x.size() || j < y.size()) {
    if (j == y.size() || (i < x.size() && x[i] < y[j])) out.push_back(x[i++]);
    else if (i == x.size() || y[j] < x[i]) out.push_back(y[j++]);
    else { i++; j++; }
  }
  return out;
}
struct Word { Lin bit[32]; };
static Word word_slot(int base) { Word w; for (int i = 0; i < 32; i++) w.bit[i] = {(uint32_t)(base + i)}; return w; }
static Word word_const(uint32_t v) { Word w; for (int i = 0; i < 32; i++) if ((v >> i) & 1) w.bit[i] = {(uint32_t)Z_CONST_POS}; return w; }
static Word word_xor(const Word& x, const Word& y) { Word w; for (int i = 0; i < 32; i++) w.bit[i] = lin_xor(x.bit[i], y.bit[i]); return w; }
static Word word_rotr(const Word& x, int n) { Word w; for (int i = 0; i < 32; i++) w.bit[i] = x.bit[(i + n) % 32]; return w; }

// Carry rows of x + y and the symbolic sum (blake3.rs:418-448, :402-416).
static Word add_rows(SparseRows& A, SparseRows& B, const Word& x, const Word& y, int base) {
  Lin prefix;  // carry[0..i)
  Word sum;
  for (int i = 0; i < 32; i++) {
    if (i < 31) {
      A.rows[base + i] = lin_xor(x.bit[i], prefix);
      B.rows[base + i] = lin_xor(y.bit[i], prefix);
    }
    sum.bit[i] = lin_xor(lin_xor(x.bit[i], y.bit[i]), prefix);
    if (i < 31) prefix.push_back((uint32_t)(base + i));  // indices ascend
  }
  return sum;
}

void build_matrices(SparseRows& A, SparseRows& B) {
  static int sched[7][8][2];
  msg_schedule(sched);
  A.rows.assign(K, {});
  B.rows.assign(K, {});
  A.rows[Z_CONST_POS] = {(uint32_t)Z_CONST_POS};
  B.rows[Z_CONST_POS] = {(uint32_t)Z_CONST_POS};
  auto input = [&](int base, int len) {
    for (int j = 0; j < len; j++) {
      A.rows[base + j] = {(uint32_t)(base + j)};
      B.rows[base + j] = {(uint32_t)Z_CONST_POS};
    }
  };
  input(CV_BASE, 256);
  input(M_BASE, 512);
  input(T_LO_BASE, 32);
  input(T_HI_BASE, 32);
  input(BLEN_BASE, 32);
  input(FLAGS_BASE, 32);
  Word st[16];
  for (int w = 0; w < 8; w++) st[w] = word_slot(CV_BASE + 32 * w);
  for (int i = 0; i < 4; i++) st[8 + i] = word_const(B3_IV[i]);
  st[12] = word_slot(T_LO_BASE);
  st[13] = word_slot(T_HI_BASE);
  st[14] = word_slot(BLEN_BASE);
  st[15] = word_slot(FLAGS_BASE);
  for (int r = 0; r < 7; r++) {
    for (int gi = 0; gi < 8; gi++) {
      int g = r * 8 + gi;
      const int* L = G_LANES[gi];
      Word a = st[L[0]], b = st[L[1]], c = st[L[2]], d = st[L[3]];
      Word mx = word_slot(M_BASE + 32 * sched[r][gi][0]);
      Word my = word_slot(M_BASE + 32 * sched[r][gi][1]);
      Word tmp0 = add_rows(A, B, a, b, carry_base(g, 0));
      Word a1 = add_rows(A, B, tmp0, mx, carry_base(g, 1));
      Word d1 = word_rotr(word_xor(d, a1), 16);
      Word c1 = add_rows(A, B, c, d1, carry_base(g, 2));
      Word b1 = word_rotr(word_xor(b, c1), 12);
      Word tmp1 = add_rows(A, B, a1, b1, carry_base(g, 3));
      Word a2 = add_rows(A, B, tmp1, my, carry_base(g, 4));
      Word d2 = word_rotr(word_xor(d1, a2), 8);
      Word c2 = add_rows(A, B, c1, d2, carry_base(g, 5));
      Word bn = word_rotr(word_xor(b1, c2), 7);
      for (int i = 0; i < 32; i++) {
        A.rows[lin_base(g, 0) + i] = bn.bit[i];
        B.rows[lin_base(g, 0) + i] = {(uint32_t)Z_CONST_POS};
        A.rows[lin_base(g, 1) + i] = d2.bit[i];
        B.rows[lin_base(g, 1) + i] = {(uint32_t)Z_CONST_POS};
      }
      st[L[0]] = a2;
      st[L[1]] = word_slot(lin_base(g, 0));
      st[L[2]] = c2;
      st[L[3]] = word_slot(lin_base(g, 1));
    }
  }
  for (int w = 0; w < 8; w++) {
    Word lo = word_xor(st[w], st[w + 8]);
    Word hi = word_xor(st[w + 8], word_slot(CV_BASE + 32 * w));
    for (int i = 0; i < 32; i++) {
      A.rows[OUT_LO_BASE + 32 * w + i] = lo.bit[i];
      B.rows[OUT_LO_BASE + 32 * w + i] = {(uint32_t)Z_CONST_POS};
      A.rows[OUT_HI_BASE + 32 * w + i] = hi.bit[i];
      B.rows[OUT_HI_BASE + 32 * w + i] = {(uint32_t)Z_CONST_POS};
    }
  }
}

// r1cs.rs:343-365 and the length-prefixed matrix absorption at :431-460.
static void absorb_u64(Blake3& h, uint64_t v) {
  uint8_t b[8];
  for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (8 * i));
  h.update(b, 8);
}
static void absorb_rows(Blake3& h, const SparseRows& M) {
  absorb_u64(h, K);
  absorb_u64(h, K);
  std::vector<uint8_t> buf;
  for (const auto& row : M.rows) {
    buf.resize(8 * (row.size() + 1));
    uint64_t n = row.size();
    for (int i = 0; i < 8; i++) buf[i] = (uint8_t)(n >> (8 * i));
    for (size_t j = 0; j < row.size(); j++)
      for (int i = 0; i < 8; i++) buf[8 * (j + 1) + i] = (uint8_t)((uint64_t)row[j] >> (8 * i));
    h.update(buf.data(), buf.size());
  }
}

void statement_digest(int m, const SparseRows& A, const SparseRows& B, uint8_t out[32]) {
  Blake3 h;
  const char* label = "flock-r1cs-stmt-v1";
  h.update(label, strlen(label));
  absorb_u64(h, (uint64_t)m);
  absorb_u64(h, K_LOG);
  absorb_u64(h, K_SKIP);
  uint8_t layout = 0;  // WitnessLayout::RowMajor
  h.update(&layout, 1);
  absorb_rows(h, A);
  absorb_rows(h, B);
  SparseRows C;
  C.rows.resize(K);
  for (int i = 0; i < K; i++) C.rows[i] = {(uint32_t)i};
  absorb_rows(h, C);
  h.finalize(out);
}

}  // namespace oracle
