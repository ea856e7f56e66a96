// Additive NTT, Merkle tree and PCS commit for the oracle (test infrastructure only).
#include <algorithm>
#include <cstring>

#include "oracle.h"

namespace oracle {

// Normalized subspace-polynomial evaluations and the breadth-first twiddle
// table: crates/flock-core/src/ntt/additive_ntt_f128.rs:57-88 and :106-129,
// with the standard basis {1, x, ..., x^(dim-1)} of :514-522.
NttF128::NttF128(int dim) : log_d(dim) {
  std::vector<std::vector<F128>> evals;
  std::vector<F128> basis(dim);
  for (int i = 0; i < dim; i++) basis[i] = i < 64 ? f128(1ULL << i, 0) : f128(0, 1ULL << (i - 64));
  evals.push_back(basis);
  for (int i = 1; i < dim; i++) {
    const auto& prev = evals[i - 1];
    std::vector<F128> row;
    for (size_t k = 1; k < prev.size(); k++) row.push_back(prev[k] * (prev[k] + prev[0]));
    evals.push_back(row);
  }
  for (auto& row : evals) {
    F128 inv = gf_inv(row[0]);
    for (auto& v : row) v = v * inv;
  }
  twiddles.clear();
  for (int layer = 0; layer < dim; layer++) {
    size_t start = twiddles.size();
    const auto& row = evals[dim - layer - 1];
    twiddles.push_back(F128());
    for (size_t bit = 0; bit + 1 < row.size(); bit++) {
      size_t half = (size_t)1 << bit;
      for (size_t b = 0; b < half; b++) twiddles.push_back(twiddles[start + b] + row[bit + 1]);
    }
  }
}

// Scalar interleaved transform, additive_ntt_f128.rs:1281-1312.
void NttF128::forward_interleaved(F128* data, size_t n_total, size_t num_ntts, int start_layer) const {
  size_t n = n_total / num_ntts;
  int ld = 0;
  while (((size_t)1 << ld) < n) ld++;
  for (int layer = start_layer; layer < ld; layer++) {
    size_t num_blocks = (size_t)1 << layer;
    size_t half = (size_t)1 << (ld - layer - 1);
    // one work item per (block, row) pair; all pairs of a layer are independent
#pragma omp parallel for schedule(static) if (num_blocks * half >= 4096)
    for (int64_t item = 0; item < (int64_t)(num_blocks * half); item++) {
      size_t blk = (size_t)item / half, row = (size_t)item % half;
      F128 t = twiddle(layer, blk);
      size_t base = blk * 2 * half * num_ntts;
      {
        F128* top = data + base + row * num_ntts;
        F128* bot = top + half * num_ntts;
        for (size_t lane = 0; lane < num_ntts; lane++) {
          F128 v = bot[lane];
          F128 u = top[lane] + v * t;
          top[lane] = u;
          bot[lane] = v + u;
        }
      }
    }
  }
}

bool Hash32::operator==(const Hash32& o) const { return memcmp(b, o.b, 32) == 0; }

// merkle.rs:200-210: leaf = non-root chaining value of the leaf bytes,
// parent = PARENT-flag compression of left||right.
Hash32 leaf_cv(const uint8_t* data, size_t len) {
  Blake3 h;
  h.update(data, len);
  Hash32 out;
  h.finalize_non_root(out.b);
  return out;
}
Hash32 parent_cv(const Hash32& l, const Hash32& r) {
  Hash32 out;
  b3_parent_cv(l.b, r.b, out.b);
  return out;
}

// merkle.rs:816-839 (sequential tree, flat layout).
std::vector<Hash32> merkle_tree(const uint8_t* data, size_t len, size_t n_leaves) {
  size_t leaf = len / n_leaves;
  std::vector<Hash32> tree(2 * n_leaves - 1);
#pragma omp parallel for schedule(static) if (n_leaves >= 256)
  for (int64_t i = 0; i < (int64_t)n_leaves; i++) tree[i] = leaf_cv(data + i * leaf, leaf);
  size_t rs = 0, rl = n_leaves;
  while (rl > 1) {
    size_t nl = rl / 2;
#pragma omp parallel for schedule(static) if (nl >= 1024)
    for (int64_t i = 0; i < (int64_t)nl; i++) tree[rs + rl + i] = parent_cv(tree[rs + 2 * i], tree[rs + 2 * i + 1]);
    rs += rl;
    rl = nl;
  }
  return tree;
}

// merkle.rs:879-928 (octopus multi-proof).
std::vector<Hash32> merkle_multi_proof(const std::vector<Hash32>& tree, size_t n_leaves,
                                       std::vector<size_t> active) {
  std::vector<Hash32> proof;
  if (active.empty() || n_leaves == 1) return proof;
  std::sort(active.begin(), active.end());
  active.erase(std::unique(active.begin(), active.end()), active.end());
  size_t ls = 0, ll = n_leaves;
  while (ll > 1) {
    std::vector<size_t> next;
    size_t i = 0;
    while (i < active.size()) {
      size_t p = active[i];
      bool sib = i + 1 < active.size() && active[i + 1] == (p ^ 1);
      if (sib) i += 2;
      else { proof.push_back(tree[ls + (p ^ 1)]); i += 1; }
      next.push_back(p >> 1);
    }
    active = next;
    ls += ll;
    ll >>= 1;
  }
  return proof;
}

// merkle.rs:937-1004
bool verify_merkle_multi_proof(const Hash32& root, size_t n_leaves, const std::vector<size_t>& pos,
                               const std::vector<Hash32>& leaves, const std::vector<Hash32>& proof) {
  if (n_leaves == 0 || (n_leaves & (n_leaves - 1))) return false;
  if (pos.size() != leaves.size()) return false;
  if (pos.empty()) return proof.empty();
  for (size_t i = 0; i < pos.size(); i++) {
    if (pos[i] >= n_leaves) return false;
    if (i > 0 && pos[i - 1] >= pos[i]) return false;
  }
  if (n_leaves == 1) return proof.empty() && leaves[0] == root;
  std::vector<std::pair<size_t, Hash32>> active;
  for (size_t i = 0; i < pos.size(); i++) active.push_back({pos[i], leaves[i]});
  size_t pi = 0, ll = n_leaves;
  while (ll > 1) {
    std::vector<std::pair<size_t, Hash32>> next;
    size_t i = 0;
    while (i < active.size()) {
      size_t p = active[i].first;
      Hash32 h = active[i].second;
      bool sib = i + 1 < active.size() && active[i + 1].first == (p ^ 1);
      Hash32 l, r;
      if (sib) { l = h; r = active[i + 1].second; i += 2; }
      else {
        if (pi >= proof.size()) return false;
        Hash32 s = proof[pi++];
        i += 1;
        if ((p & 1) == 0) { l = h; r = s; } else { l = s; r = h; }
      }
      next.push_back({p >> 1, parent_cv(l, r)});
    }
    active = next;
    ll >>= 1;
  }
  if (pi != proof.size()) return false;
  return active.size() == 1 && active[0].second == root;
}

// commit.rs:250-473 + :722-818: replicate z into 2^log_inv_rate sub-blocks
// (the state after the first log_inv_rate NTT layers of [z, 0, ...]), run the
// interleaved NTT from that layer, then Merkle-hash one leaf per position.
CommitData commit(const std::vector<F128>& z, const PcsParams& p) {
  CommitData out;
  size_t len = p.n_positions() * p.num_ntts();
  out.codeword.resize(len);
  for (size_t i = 0; i < len; i++) out.codeword[i] = z[i % z.size()];
  NttF128 ntt(p.k_code());
  ntt.forward_interleaved(out.codeword.data(), len, p.num_ntts(), p.log_inv_rate);
  out.tree = merkle_tree((const uint8_t*)out.codeword.data(), len * 16, p.n_positions());
  return out;
}

}  // namespace oracle
