// ORACLE — test infrastructure only. CPU restatement of the WHIR protocol layer:
//   ProtocolParameters                src/parameters.rs:9-24
//   whir::Config::new                 src/protocols/whir/config.rs:16-152
//   irs_commit::Config::{new,commit,open,verify}   src/protocols/irs_commit.rs:125-500, 585-630
//   matrix_commit (ArkFieldEncoder, hash_rows)     src/protocols/matrix_commit.rs:119-368
//   merkle_tree::{commit,open,verify}              src/protocols/merkle_tree.rs:64-305
//   sumcheck::Config::{prove,verify}               src/protocols/sumcheck.rs:46-237
//   proof_of_work::{threshold,prove,verify}        src/protocols/proof_of_work.rs:29-191
//   challenge_indices / geometric_challenge        challenge_indices.rs:6-50, geometric_challenge.rs:10-24
//   whir::Config::prove / verify, FinalClaim       whir/prover.rs:50-315, whir/verifier.rs:45-265, whir/mod.rs:63-74
// Only mask_length == 0 (non-ZK WHIR) is restated; the ZK variant is out of scope.
#pragma once
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "algebra.hpp"
#include "hashes.hpp"
#include "transcript.hpp"

namespace oracle {

struct Digest {
  uint8_t b[32];
  bool operator==(const Digest& o) const { return memcmp(b, o.b, 32) == 0; }
  bool operator!=(const Digest& o) const { return !(*this == o); }
};

struct ProtocolParameters {
  bool unique_decoding;
  size_t starting_log_inv_rate;
  size_t initial_folding_factor;
  size_t folding_factor;
  size_t security_level;
  size_t pow_bits;
  size_t batch_size;
  uint8_t hash_id[32];
};

static constexpr double LOG2_10 = 3.32192809488736234787031942948939018;

// ------------------------------------------------------------------------------------------
// Base-field byte codecs
// ------------------------------------------------------------------------------------------
template <class B>
inline void base_to_bytes(const B& x, uint8_t* out) {
  constexpr int N = PrimeInfo<B>::N;
  uint64_t l[N];
  x.to_limbs(l);
  int nb = PrimeInfo<B>::bytes();
  for (int i = 0; i < nb; ++i) out[i] = (uint8_t)(l[i / 8] >> (8 * (i % 8)));
}

template <class B>
inline B base_from_bytes_mod(const uint8_t* b, size_t n) {
  B acc = B::zero();
  uint64_t two64_l[PrimeInfo<B>::N] = {0};
  B two64;
  if (PrimeInfo<B>::N == 1) {
    two64 = B::from_u64(GL_EPS);  // Goldilocks: 2^64 mod p
  } else {
    two64_l[1] = 1;
    two64 = B::from_limbs(two64_l);
  }
  size_t words = (n + 7) / 8;
  for (size_t w = words; w-- > 0;) {
    uint64_t x = 0;
    for (int i = 7; i >= 0; --i) {
      size_t k = w * 8 + i;
      x = (x << 8) | (k < n ? b[k] : 0);
    }
    B xv;
    if (PrimeInfo<B>::N == 1) {
      xv = B::from_u64(x);
    } else {
      uint64_t l[PrimeInfo<B>::N] = {0};
      l[0] = x;
      xv = B::from_limbs(l);
    }
    acc = acc * two64 + xv;
  }
  return acc;
}

template <class F>
inline size_t elem_bytes() {
  return (size_t)F::DEG * PrimeInfo<typename F::Base>::bytes();
}
template <class F>
inline void elem_to_bytes(const F& x, uint8_t* out) {
  typedef typename F::Base B;
  int nb = PrimeInfo<B>::bytes();
  for (int d = 0; d < F::DEG; ++d) base_to_bytes<B>(x.coeff(d), out + d * nb);
}
template <class F>
inline F elem_from_bytes_exact(const uint8_t* in, bool* ok) {
  typedef typename F::Base B;
  constexpr int N = PrimeInfo<B>::N;
  int nb = PrimeInfo<B>::bytes();
  B c[F::DEG];
  for (int d = 0; d < F::DEG; ++d) {
    uint64_t l[N] = {0};
    for (int i = 0; i < nb; ++i) l[i / 8] |= (uint64_t)in[d * nb + i] << (8 * (i % 8));
    if (!B::limbs_valid(l)) *ok = false;
    c[d] = B::from_limbs(l);
  }
  return F::from_coeffs(c);
}

// Element <-> canonical ABI limbs (DEG * N u64 per element).
template <class F>
inline void elem_to_limbs(const F& x, uint64_t* out) {
  typedef typename F::Base B;
  constexpr int N = PrimeInfo<B>::N;
  for (int d = 0; d < F::DEG; ++d) x.coeff(d).to_limbs(out + d * N);
}
template <class F>
inline F elem_from_limbs(const uint64_t* in) {
  typedef typename F::Base B;
  constexpr int N = PrimeInfo<B>::N;
  B c[F::DEG];
  for (int d = 0; d < F::DEG; ++d) c[d] = B::from_limbs(in + d * N);
  return F::from_coeffs(c);
}
template <class F>
inline bool elem_limbs_valid(const uint64_t* in) {
  typedef typename F::Base B;
  constexpr int N = PrimeInfo<B>::N;
  for (int d = 0; d < F::DEG; ++d)
    if (!B::limbs_valid(in + d * N)) return false;
  return true;
}
template <class F>
inline constexpr int elem_limbs() {
  return F::DEG * PrimeInfo<typename F::Base>::N;
}

template <class F>
double field_size_bits() {
  typedef typename F::Base B;
  double m = 0.0;
  uint64_t p[PrimeInfo<B>::N];
  PrimeInfo<B>::pm1(p);
  p[0] += 1;
  for (int i = PrimeInfo<B>::N - 1; i >= 0; --i) m = m * 18446744073709551616.0 + (double)p[i];
  return std::log2(m) * (double)F::DEG;
}

// ------------------------------------------------------------------------------------------
// Transcript helpers
// ------------------------------------------------------------------------------------------
template <class F, class St>
void send_elem(St& ps, const F& x) {
  std::vector<uint8_t> b(elem_bytes<F>());
  elem_to_bytes<F>(x, b.data());
  ps.prover_bytes(b.data(), b.size());
}
template <class F>
F recv_elem(VerifierState& vs) {
  std::vector<uint8_t> b(elem_bytes<F>());
  vs.prover_bytes(b.data(), b.size());
  bool ok = true;
  F x = elem_from_bytes_exact<F>(b.data(), &ok);
  if (!ok) throw VerificationError();
  return x;
}
template <class F, class St>
F challenge_elem(St& st) {
  typedef typename F::Base B;
  size_t nb = PrimeInfo<B>::bytes() + 16;
  B c[F::DEG];
  std::vector<uint8_t> buf(nb);
  for (int d = 0; d < F::DEG; ++d) {
    st.verifier_bytes(buf.data(), nb);
    c[d] = base_from_bytes_mod<B>(buf.data(), nb);
  }
  return F::from_coeffs(c);
}
template <class F, class St>
std::vector<F> geometric_challenge(St& st, size_t count) {
  if (count == 0) return {};
  if (count == 1) return {F::one()};
  F x = challenge_elem<F>(st);
  std::vector<F> r(count);
  r[0] = F::one();
  for (size_t i = 1; i < count; ++i) r[i] = r[i - 1] * x;
  return r;
}
template <class St>
std::vector<size_t> challenge_indices(St& st, size_t num_leaves, size_t count, bool dedup) {
  if (count == 0) return {};
  if (num_leaves == 0 || (num_leaves & (num_leaves - 1))) throw std::runtime_error("num_leaves must be a power of two");
  if (num_leaves == 1) return dedup ? std::vector<size_t>{0} : std::vector<size_t>(count, 0);
  size_t log = 0;
  while (((size_t)1 << log) < num_leaves) ++log;
  size_t sb = (log + 7) / 8;
  std::vector<uint8_t> ent(count * sb);
  st.verifier_bytes(ent.data(), ent.size());
  std::vector<size_t> idx(count);
  for (size_t i = 0; i < count; ++i) {
    size_t acc = 0;
    for (size_t k = 0; k < sb; ++k) acc = (acc << 8) | ent[i * sb + k];
    idx[i] = acc % num_leaves;
  }
  if (dedup) {
    std::sort(idx.begin(), idx.end());
    idx.erase(std::unique(idx.begin(), idx.end()), idx.end());
  }
  return idx;
}

// ------------------------------------------------------------------------------------------
// Proof of work
// ------------------------------------------------------------------------------------------
struct PowConfig {
  uint8_t hash_id[32];
  uint64_t threshold;
};

inline uint64_t pow_threshold(double bits) {
  if (!(bits >= 0.0 && bits <= 60.0)) throw std::runtime_error("pow difficulty out of range [0, 60]");
  double t = std::ceil(std::exp2(64.0 - bits));
  if (t >= 18446744073709551615.0) return UINT64_MAX;
  return (uint64_t)t;
}
inline double pow_difficulty(uint64_t threshold) { return 64.0 - std::log2((double)threshold); }

// Lowest nonce with LE-u64(H(challenge || nonce_le || 0^24)[0..8]) <= threshold.
uint64_t pow_grind(HashKind kind, const uint8_t challenge[32], uint64_t threshold);

template <class St>
void pow_prove(const PowConfig& c, St& ps) {
  if (c.threshold == UINT64_MAX) return;
  HashKind k = hash_kind(c.hash_id);
  if (k == HK_INVALID) throw std::runtime_error("Hash Engine not found");
  uint8_t chal[32];
  ps.verifier_bytes(chal, 32);
  uint64_t nonce = pow_grind(k, chal, c.threshold);
  uint8_t nb[8];
  for (int i = 0; i < 8; ++i) nb[i] = (uint8_t)(nonce >> (8 * i));
  ps.prover_bytes(nb, 8);
}
inline void pow_verify(const PowConfig& c, VerifierState& vs) {
  if (c.threshold == UINT64_MAX) return;
  HashKind k = hash_kind(c.hash_id);
  if (k == HK_INVALID) throw VerificationError();
  uint8_t chal[32], nb[8], in[64] = {0}, out[32];
  vs.verifier_bytes(chal, 32);
  vs.prover_bytes(nb, 8);
  memcpy(in, chal, 32);
  memcpy(in + 32, nb, 8);
  if (hash_many(k, 64, in, 1, out)) throw VerificationError();
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | out[i];
  if (v > c.threshold) throw VerificationError();
}

// ------------------------------------------------------------------------------------------
// Merkle tree + matrix commitment
// ------------------------------------------------------------------------------------------
inline size_t layers_for_size(size_t n) {
  size_t p = next_pow2(n == 0 ? 1 : n), l = 0;
  while (((size_t)1 << l) < p) ++l;
  return n == 0 ? 0 : l;
}

struct MerkleConfig {
  size_t num_leaves;
  size_t layers;
  uint8_t hash_id[32];
  size_t num_nodes() const { return ((size_t)1 << (layers + 1)) - 1; }
};

// Nodes: [leaves padded to 2^layers][next layer]...[root]
std::vector<Digest> merkle_build(const MerkleConfig& c, const std::vector<Digest>& leaves);
// Sibling hints for sorted/deduplicated indices, in the order merkle_tree.rs:145-186 writes them.
std::vector<Digest> merkle_open_hints(const MerkleConfig& c, const std::vector<Digest>& nodes,
                                      const std::vector<size_t>& indices);
// merkle_tree.rs:188-273; throws VerificationError on mismatch.
void merkle_verify(const MerkleConfig& c, VerifierState& vs, const Digest& root, const std::vector<size_t>& indices,
                   const std::vector<Digest>& leaf_hashes);

// Row-wise leaf digests of a row-major matrix (matrix_commit.rs:311-368, ArkFieldEncoder 130-156).
template <class F>
std::vector<Digest> hash_rows(HashKind kind, const F* matrix, size_t rows, size_t cols) {
  std::vector<Digest> out(rows);
  size_t eb = elem_bytes<F>();
  size_t msg = eb * cols;
  parallel_for(rows, 256, [&](size_t s, size_t e) {
    std::vector<uint8_t> buf(msg ? msg : 1);
    for (size_t r = s; r < e; ++r) {
      for (size_t c = 0; c < cols; ++c) elem_to_bytes<F>(matrix[r * cols + c], buf.data() + c * eb);
      if (hash_many(kind, msg, buf.data(), 1, out[r].b)) throw std::runtime_error("hash engine does not support size");
    }
  });
  return out;
}

// ------------------------------------------------------------------------------------------
// Configuration (irs_commit.rs:125-288, whir/config.rs:16-152)
// ------------------------------------------------------------------------------------------
struct IrsConfig {
  size_t num_vectors, vector_size, mask_length, codeword_length, interleaving_depth;
  size_t num_cols;  // matrix_commit.num_cols
  uint8_t leaf_hash_id[32];
  MerkleConfig merkle;
  double johnson_slack;
  size_t in_domain_samples, out_domain_samples;
  bool deduplicate_in_domain;
  double field_bits;  // target field size in bits

  size_t message_length() const { return vector_size / interleaving_depth; }
  size_t masked_message_length() const { return message_length() + mask_length; }
  size_t num_messages() const { return interleaving_depth * num_vectors; }
  double rate() const { return (double)masked_message_length() / (double)codeword_length; }
  bool unique_decoding() const { return out_domain_samples == 0 && johnson_slack == 0.0; }
  double list_size() const {
    if (unique_decoding()) return 1.0;
    return 1. / (2. * johnson_slack * std::sqrt(rate()));
  }
  double rbr_ood_sample() const {
    double L = list_size();
    double l_choose_2 = L * (L - 1.) / 2.;
    double log_per_sample = std::log2((double)(vector_size - 1)) - field_bits;
    return -std::log2(l_choose_2) - (double)out_domain_samples * log_per_sample;
  }
  double rbr_queries() const {
    double per_sample = unique_decoding() ? (1. + rate()) / 2. : std::sqrt(rate()) + johnson_slack;
    return (double)in_domain_samples * -std::log2(per_sample);
  }
  double rbr_soundness_fold_prox_gaps() const {
    double log_inv_rate = -std::log2(rate());
    double log_k = std::log2((double)masked_message_length());
    double error;
    if (unique_decoding()) {
      error = log_k + log_inv_rate;
    } else {
      error = 7. * LOG2_10 + 3.5 * log_inv_rate + 2. * log_k;
    }
    return field_bits - error;
  }
};

IrsConfig irs_config_new(double security_target, bool unique_decoding, const uint8_t hash_id[32], size_t num_vectors,
                         size_t vector_size, size_t interleaving_depth, double rate, double field_bits);

struct SumcheckConfig {
  size_t initial_size;
  PowConfig round_pow;
  size_t num_rounds;
  size_t mask_length;
  size_t final_size() const {
    if (initial_size == 0 || num_rounds == 0) return initial_size;
    return next_pow2(initial_size) >> num_rounds;
  }
};

struct RoundConfig {
  IrsConfig irs;
  SumcheckConfig sumcheck;
  PowConfig pow;
};

struct WhirConfig {
  IrsConfig initial_committer;
  SumcheckConfig initial_sumcheck;
  PowConfig initial_skip_pow;
  std::vector<RoundConfig> rounds;
  SumcheckConfig final_sumcheck;
  PowConfig final_pow;
  size_t initial_size() const { return initial_committer.vector_size; }
};

WhirConfig whir_config_new(size_t size, const ProtocolParameters& p, double field_bits);
// Canonical byte string identifying the configuration (hashed into the protocol id).
std::vector<uint8_t> config_bytes(const WhirConfig& c, int field_kind);
std::string config_json(const WhirConfig& c);

// ------------------------------------------------------------------------------------------
// Interleaved RS commitment
// ------------------------------------------------------------------------------------------
template <class S, class T>
struct IrsWitness {
  std::vector<S> matrix;  // codeword_length x num_cols, row major
  std::vector<Digest> nodes;
  std::vector<T> ood_points;
  std::vector<T> ood_matrix;  // ood_points x num_vectors
  size_t num_vectors() const { return ood_points.empty() ? 0 : ood_matrix.size() / ood_points.size(); }
};

template <class S>
struct InDomain {
  std::vector<S> points;
  std::vector<S> matrix;  // points x stride
  size_t cols() const { return points.empty() ? 0 : matrix.size() / points.size(); }
};

template <class S, class T>
IrsWitness<S, T> irs_commit(const IrsConfig& c, ProverState& ps, const std::vector<const S*>& vectors) {
  if (vectors.size() != c.num_vectors) throw std::runtime_error("wrong number of vectors");
  IrsWitness<S, T> w;
  size_t L = c.message_length();
  std::vector<const S*> msgs;
  for (const S* v : vectors)
    for (size_t j = 0; j < c.interleaving_depth; ++j) msgs.push_back(v + j * L);
  w.matrix = interleaved_encode<S>(msgs, L, nullptr, 0, c.codeword_length);
  HashKind lk = hash_kind(c.leaf_hash_id);
  if (lk == HK_INVALID) throw std::runtime_error("unknown leaf hash");
  std::vector<Digest> leaves = hash_rows<S>(lk, w.matrix.data(), c.codeword_length, c.num_cols);
  w.nodes = merkle_build(c.merkle, leaves);
  ps.prover_bytes(w.nodes.back().b, 32);
  for (size_t i = 0; i < c.out_domain_samples; ++i) w.ood_points.push_back(challenge_elem<T>(ps));
  for (const T& pt : w.ood_points) {
    for (const S* v : vectors) {
      T val = univariate_evaluate<T, S>(v, c.vector_size, pt);
      send_elem<T>(ps, val);
      w.ood_matrix.push_back(val);
    }
  }
  return w;
}

template <class S, class T>
struct IrsCommitment {
  Digest root;
  std::vector<T> ood_points;
  std::vector<T> ood_matrix;
  size_t num_vectors() const { return ood_points.empty() ? 0 : ood_matrix.size() / ood_points.size(); }
};

template <class S, class T>
IrsCommitment<S, T> irs_receive(const IrsConfig& c, VerifierState& vs) {
  IrsCommitment<S, T> cm;
  vs.prover_bytes(cm.root.b, 32);
  for (size_t i = 0; i < c.out_domain_samples; ++i) cm.ood_points.push_back(challenge_elem<T>(vs));
  for (size_t i = 0; i < c.out_domain_samples * c.num_vectors; ++i) cm.ood_matrix.push_back(recv_elem<T>(vs));
  return cm;
}

template <class S>
void hint_rows(ProverState& ps, const std::vector<S>& rows) {
  uint8_t lb[8];
  uint64_t n = rows.size();
  for (int i = 0; i < 8; ++i) lb[i] = (uint8_t)(n >> (8 * i));
  ps.hint_bytes(lb, 8);
  std::vector<uint8_t> b(elem_bytes<S>());
  for (const S& x : rows) {
    elem_to_bytes<S>(x, b.data());
    ps.hint_bytes(b.data(), b.size());
  }
}

template <class S, class T>
InDomain<S> irs_open(const IrsConfig& c, ProverState& ps, const std::vector<const IrsWitness<S, T>*>& ws) {
  std::vector<size_t> idx = challenge_indices(ps, c.codeword_length, c.in_domain_samples, c.deduplicate_in_domain);
  InDomain<S> res;
  {
    std::vector<typename S::Base> pts = evaluation_points<typename S::Base>(c.masked_message_length(), c.codeword_length, idx);
    for (auto& p : pts) res.points.push_back(S::from_base(p));
  }
  size_t nc = c.num_cols;
  size_t stride = ws.size() * nc;
  res.matrix.assign(idx.size() * stride, S::zero());
  size_t off = 0;
  std::vector<size_t> sorted = idx;
  std::sort(sorted.begin(), sorted.end());
  sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
  for (const IrsWitness<S, T>* w : ws) {
    std::vector<S> sub;
    for (size_t pi = 0; pi < idx.size(); ++pi) {
      for (size_t k = 0; k < nc; ++k) {
        S v = w->matrix[idx[pi] * nc + k];
        sub.push_back(v);
        res.matrix[pi * stride + off + k] = v;
      }
    }
    hint_rows<S>(ps, sub);
    std::vector<Digest> hints = merkle_open_hints(c.merkle, w->nodes, sorted);
    for (auto& h : hints) ps.hint_bytes(h.b, 32);
    off += nc;
  }
  return res;
}

template <class S, class T>
InDomain<S> irs_verify(const IrsConfig& c, VerifierState& vs, const std::vector<const IrsCommitment<S, T>*>& cms) {
  for (auto* cm : cms) {
    if (cm->ood_points.size() != c.out_domain_samples) throw VerificationError();
    if (cm->ood_matrix.size() != c.num_vectors * c.out_domain_samples) throw VerificationError();
  }
  std::vector<size_t> idx = challenge_indices(vs, c.codeword_length, c.in_domain_samples, c.deduplicate_in_domain);
  InDomain<S> res;
  {
    std::vector<typename S::Base> pts = evaluation_points<typename S::Base>(c.masked_message_length(), c.codeword_length, idx);
    for (auto& p : pts) res.points.push_back(S::from_base(p));
  }
  size_t nc = c.num_cols;
  size_t stride = cms.size() * nc;
  res.matrix.assign(idx.size() * stride, S::zero());
  size_t off = 0;
  HashKind lk = hash_kind(c.leaf_hash_id);
  if (lk == HK_INVALID) throw VerificationError();
  for (auto* cm : cms) {
    uint8_t lb[8];
    vs.hint_bytes(lb, 8);
    uint64_t n = 0;
    for (int i = 7; i >= 0; --i) n = (n << 8) | lb[i];
    if (n != idx.size() * nc) throw VerificationError();
    std::vector<S> sub(n);
    std::vector<uint8_t> b(elem_bytes<S>());
    for (uint64_t i = 0; i < n; ++i) {
      vs.hint_bytes(b.data(), b.size());
      bool ok = true;
      sub[i] = elem_from_bytes_exact<S>(b.data(), &ok);
      if (!ok) throw VerificationError();
    }
    std::vector<Digest> leaf = hash_rows<S>(lk, sub.data(), idx.size(), nc);
    merkle_verify(c.merkle, vs, cm->root, idx, leaf);
    for (size_t pi = 0; pi < idx.size(); ++pi)
      for (size_t k = 0; k < nc; ++k) res.matrix[pi * stride + off + k] = sub[pi * nc + k];
    off += nc;
  }
  return res;
}

// ------------------------------------------------------------------------------------------
// Sumcheck protocol (mask_length == 0)
// ------------------------------------------------------------------------------------------
template <class F>
std::vector<F> sumcheck_prove(const SumcheckConfig& c, ProverState& ps, std::vector<F>& a, std::vector<F>& b, F& sum) {
  if (c.mask_length != 0) throw std::runtime_error("masked sumcheck is out of scope");
  if (a.size() != c.initial_size || b.size() != c.initial_size) throw std::runtime_error("sumcheck size mismatch");
  std::vector<F> rs;
  bool have_prev = false;
  F prev = F::zero();
  for (size_t round = 0; round < c.num_rounds; ++round) {
    F c0, c2;
    if (have_prev) {
      fold(a, prev);
      fold(b, prev);
    }
    compute_sumcheck_polynomial(a, b, &c0, &c2);
    F c1 = sum - c0.dbl() - c2;
    send_elem<F>(ps, c0);
    send_elem<F>(ps, c2);
    pow_prove(c.round_pow, ps);
    F r = challenge_elem<F>(ps);
    rs.push_back(r);
    sum = (c2 * r + c1) * r + c0;
    prev = r;
    have_prev = true;
  }
  if (have_prev) {
    fold(a, prev);
    fold(b, prev);
  }
  return rs;
}

template <class F>
std::vector<F> sumcheck_verify(const SumcheckConfig& c, VerifierState& vs, F& sum) {
  std::vector<F> rs;
  for (size_t round = 0; round < c.num_rounds; ++round) {
    F u0 = recv_elem<F>(vs);
    F u2 = recv_elem<F>(vs);
    F u1 = sum - u0.dbl() - u2;
    pow_verify(c.round_pow, vs);
    F r = challenge_elem<F>(vs);
    rs.push_back(r);
    sum = (u2 * r + u1) * r + u0;  // univariate_evaluate([u0,u1,u2], r) by Horner
  }
  return rs;
}

// ------------------------------------------------------------------------------------------
// Linear forms used as statements: multilinear-extension evaluations and explicit covectors.
// ------------------------------------------------------------------------------------------
template <class T>
struct LinearForms {
  std::vector<std::vector<T>> mle_points;  // each num_variables long
  std::vector<std::vector<T>> covectors;   // each size long
  size_t count() const { return mle_points.size() + covectors.size(); }
};

template <class T>
T mle_of_eq(const std::vector<T>& l, const std::vector<T>& r) {
  T acc = T::one();
  for (size_t i = 0; i < l.size(); ++i) acc = acc * (l[i] * r[i] + (T::one() - l[i]) * (T::one() - r[i]));
  return acc;
}

template <class T>
T univariate_mle(const T& x, const std::vector<T>& point) {
  // univariate_evaluation.rs:44-53 (point consumed in reverse order)
  T x2i = x, res = T::one();
  for (size_t k = point.size(); k-- > 0;) {
    const T& r = point[k];
    res = res * ((T::one() - r) + r * x2i);
    x2i = x2i * x2i;
  }
  return res;
}

template <class T>
struct FinalClaim {
  std::vector<T> evaluation_point;
  std::vector<T> rlc_coefficients;
  T linear_form_rlc;
};

template <class T>
std::vector<T> eq_weights(const std::vector<T>& point) {
  std::vector<T> r((size_t)1 << point.size(), T::zero());
  eval_eq(r, point, T::one());
  return r;
}
template <class T>
std::vector<T> tensor_product(const std::vector<T>& a, const std::vector<T>& b) {
  std::vector<T> r;
  for (auto& x : a)
    for (auto& y : b) r.push_back(x * y);
  return r;
}
template <class T>
T dot(const std::vector<T>& a, const std::vector<T>& b) {
  if (a.size() != b.size()) throw std::runtime_error("dot length mismatch");
  T acc = T::zero();
  for (size_t i = 0; i < a.size(); ++i) acc += a[i] * b[i];
  return acc;
}

// ------------------------------------------------------------------------------------------
// WHIR prover (whir/prover.rs:50-315). `witnesses` commit `batch_size` vectors each;
// `vectors` lists all vectors in witness order. `evaluations` is forms x vectors.
// ------------------------------------------------------------------------------------------
template <class S, class T>
FinalClaim<T> whir_prove(const WhirConfig& cfg, ProverState& ps, const std::vector<const S*>& vectors,
                         const std::vector<const IrsWitness<S, T>*>& witnesses, const LinearForms<T>& forms,
                         const std::vector<T>& evaluations) {
  size_t nv = vectors.size();
  size_t n = cfg.initial_size();
  if (nv != witnesses.size() * cfg.initial_committer.num_vectors) throw std::runtime_error("vector/witness mismatch");
  if (evaluations.size() != nv * forms.count()) throw std::runtime_error("evaluation matrix size mismatch");
  for (auto& cv : forms.covectors)
    if (cv.size() != n) throw std::runtime_error("covector size mismatch");
  for (auto& pt : forms.mle_points)
    if (((size_t)1 << pt.size()) != n) throw std::runtime_error("point size mismatch");
  FinalClaim<T> claim;
  claim.linear_form_rlc = T::zero();
  if (nv == 0) return claim;

  // OOD cross terms (prover.rs:98-128)
  std::vector<T> oods_points, oods_matrix;
  size_t voff = 0;
  for (auto* w : witnesses) {
    size_t wn = w->num_vectors();
    for (size_t oi = 0; oi < w->ood_points.size(); ++oi) {
      const T& pt = w->ood_points[oi];
      for (size_t j = 0; j < nv; ++j) {
        if (j >= voff && j < voff + wn) {
          oods_matrix.push_back(w->ood_matrix[oi * wn + (j - voff)]);
        } else {
          T e = univariate_evaluate<T, S>(vectors[j], n, pt);
          send_elem<T>(ps, e);
          oods_matrix.push_back(e);
        }
      }
      oods_points.push_back(pt);
    }
    voff += w->num_vectors();
  }

  std::vector<T> vector_rlc = geometric_challenge<T>(ps, nv);
  std::vector<T> vec(n);
  for (size_t i = 0; i < n; ++i) vec[i] = embed<T, S>(vectors[0][i]);
  for (size_t j = 1; j < nv; ++j) {
    const T& c = vector_rlc[j];
    parallel_for(n, 1 << 14, [&](size_t s, size_t e) {
      for (size_t i = s; i < e; ++i) vec[i] += c.mul_base(vectors[j][i]);
    });
  }

  size_t nforms = forms.count();
  std::vector<T> constraint_rlc = geometric_challenge<T>(ps, nforms + oods_points.size());
  bool has_constraints = !constraint_rlc.empty();
  std::vector<T> init_rlc(constraint_rlc.begin(), constraint_rlc.begin() + nforms);
  std::vector<T> oods_rlc(constraint_rlc.begin() + nforms, constraint_rlc.end());
  std::vector<T> covector;
  if (nforms > 0 || has_constraints) covector.assign(n, T::zero());
  {
    size_t k = 0;
    for (auto& pt : forms.mle_points) {
      eval_eq(covector, pt, init_rlc[k]);
      ++k;
    }
    for (auto& cv : forms.covectors) {
      const T& c = init_rlc[k];
      parallel_for(n, 1 << 14, [&](size_t s, size_t e) {
        for (size_t i = s; i < e; ++i) covector[i] += c * cv[i];
      });
      ++k;
    }
  }
  T the_sum = T::zero();
  for (size_t f = 0; f < nforms; ++f) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * evaluations[f * nv + j];
    the_sum += init_rlc[f] * row;
  }
  if (!oods_points.empty()) geometric_accumulate(covector, oods_rlc, oods_points);
  for (size_t o = 0; o < oods_points.size(); ++o) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * oods_matrix[o * nv + j];
    the_sum += oods_rlc[o] * row;
  }

  std::vector<T> folding;
  if (has_constraints) {
    folding = sumcheck_prove<T>(cfg.initial_sumcheck, ps, vec, covector, the_sum);
  } else {
    for (size_t i = 0; i < cfg.initial_sumcheck.num_rounds; ++i) folding.push_back(challenge_elem<T>(ps));
    pow_prove(cfg.initial_skip_pow, ps);
    for (auto& f : folding) fold(vec, f);
    covector.assign(cfg.initial_sumcheck.final_size(), T::zero());
  }
  std::vector<T> evaluation_point = folding;

  // Rounds
  std::unique_ptr<IrsWitness<T, T>> prev_round;
  for (size_t ri = 0; ri < cfg.rounds.size(); ++ri) {
    const RoundConfig& rc = cfg.rounds[ri];
    auto nw = std::make_unique<IrsWitness<T, T>>(irs_commit<T, T>(rc.irs, ps, std::vector<const T*>{vec.data()}));
    pow_prove(rc.pow, ps);
    InDomain<T> in_domain;
    if (!prev_round) {
      InDomain<S> d = irs_open<S, T>(cfg.initial_committer, ps, witnesses);
      for (auto& p : d.points) in_domain.points.push_back(T::from_base(p.coeff(0)));
      for (auto& x : d.matrix) in_domain.matrix.push_back(T::from_base(x.coeff(0)));
    } else {
      in_domain = irs_open<T, T>(cfg.rounds[ri - 1].irs, ps, std::vector<const IrsWitness<T, T>*>{prev_round.get()});
    }
    std::vector<T> stir_points = nw->ood_points;
    for (auto& p : in_domain.points) stir_points.push_back(p);
    std::vector<T> stir_evals;
    for (size_t o = 0; o < nw->ood_points.size(); ++o) stir_evals.push_back(nw->ood_matrix[o]);  // weights [1]
    std::vector<T> wts = tensor_product(vector_rlc, eq_weights(folding));
    size_t cols = in_domain.cols();
    for (size_t pi = 0; pi < in_domain.points.size(); ++pi) {
      std::vector<T> row(in_domain.matrix.begin() + pi * cols, in_domain.matrix.begin() + (pi + 1) * cols);
      stir_evals.push_back(dot(wts, row));
    }
    std::vector<T> stir_rlc = geometric_challenge<T>(ps, stir_points.size());
    geometric_accumulate(covector, stir_rlc, stir_points);
    the_sum += dot(stir_rlc, stir_evals);
    folding = sumcheck_prove<T>(rc.sumcheck, ps, vec, covector, the_sum);
    for (auto& f : folding) evaluation_point.push_back(f);
    prev_round = std::move(nw);
    vector_rlc = {T::one()};
  }

  if (vec.size() != cfg.final_sumcheck.initial_size) throw std::runtime_error("final vector size mismatch");
  for (auto& x : vec) send_elem<T>(ps, x);
  pow_prove(cfg.final_pow, ps);
  if (!prev_round) {
    irs_open<S, T>(cfg.initial_committer, ps, witnesses);
  } else {
    irs_open<T, T>(cfg.rounds.back().irs, ps, std::vector<const IrsWitness<T, T>*>{prev_round.get()});
  }
  std::vector<T> fin = sumcheck_prove<T>(cfg.final_sumcheck, ps, vec, covector, the_sum);
  for (auto& f : fin) evaluation_point.push_back(f);
  claim.evaluation_point = evaluation_point;
  claim.rlc_coefficients = init_rlc;
  return claim;
}

// ------------------------------------------------------------------------------------------
// WHIR verifier (whir/verifier.rs:45-265) + FinalClaim::verify (whir/mod.rs:63-74)
// ------------------------------------------------------------------------------------------
template <class S, class T>
FinalClaim<T> whir_verify(const WhirConfig& cfg, VerifierState& vs, const std::vector<const IrsCommitment<S, T>*>& cms,
                          const std::vector<T>& evaluations, size_t initial_num_variables) {
  size_t nv = cms.size() * cfg.initial_committer.num_vectors;
  FinalClaim<T> claim;
  claim.linear_form_rlc = T::zero();
  if (nv == 0) return claim;
  if (evaluations.size() % nv != 0) throw VerificationError();
  size_t nforms = evaluations.size() / nv;

  std::vector<T> oods_points, oods_matrix;
  size_t voff = 0;
  for (auto* cm : cms) {
    size_t wn = cm->num_vectors();
    for (size_t oi = 0; oi < cm->ood_points.size(); ++oi) {
      for (size_t j = 0; j < nv; ++j) {
        if (j >= voff && j < voff + wn)
          oods_matrix.push_back(cm->ood_matrix[oi * wn + (j - voff)]);
        else
          oods_matrix.push_back(recv_elem<T>(vs));
      }
      oods_points.push_back(cm->ood_points[oi]);
    }
    voff += wn;
  }
  std::vector<T> vector_rlc = geometric_challenge<T>(vs, nv);
  std::vector<T> constraint_rlc = geometric_challenge<T>(vs, oods_points.size() + nforms);
  std::vector<T> init_rlc(constraint_rlc.begin(), constraint_rlc.begin() + nforms);
  std::vector<T> oods_rlc(constraint_rlc.begin() + nforms, constraint_rlc.end());
  T the_sum = T::zero();
  for (size_t f = 0; f < nforms; ++f) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * evaluations[f * nv + j];
    the_sum += init_rlc[f] * row;
  }
  for (size_t o = 0; o < oods_points.size(); ++o) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * oods_matrix[o * nv + j];
    the_sum += oods_rlc[o] * row;
  }
  struct RoundConstraint {
    std::vector<T> rlc;
    std::vector<T> points;
    size_t size;
  };
  std::vector<RoundConstraint> constraints;
  constraints.push_back({oods_rlc, oods_points, cfg.initial_size()});
  std::vector<std::vector<T>> round_folding;
  std::vector<T> folding;
  if (constraint_rlc.empty()) {
    if (!the_sum.is_zero()) throw VerificationError();
    for (size_t i = 0; i < cfg.initial_sumcheck.num_rounds; ++i) folding.push_back(challenge_elem<T>(vs));
    pow_verify(cfg.initial_skip_pow, vs);
  } else {
    folding = sumcheck_verify<T>(cfg.initial_sumcheck, vs, the_sum);
  }
  round_folding.push_back(folding);

  std::unique_ptr<IrsCommitment<T, T>> prev;
  std::vector<T> poly_rlc;
  auto open_prev = [&](size_t ri_prev_plus1) -> InDomain<T> {
    InDomain<T> in_domain;
    if (!prev) {
      InDomain<S> d = irs_verify<S, T>(cfg.initial_committer, vs, cms);
      for (auto& p : d.points) in_domain.points.push_back(T::from_base(p.coeff(0)));
      for (auto& x : d.matrix) in_domain.matrix.push_back(T::from_base(x.coeff(0)));
      poly_rlc = vector_rlc;
    } else {
      in_domain = irs_verify<T, T>(cfg.rounds[ri_prev_plus1 - 1].irs, vs, std::vector<const IrsCommitment<T, T>*>{prev.get()});
      poly_rlc = {T::one()};
    }
    return in_domain;
  };
  for (size_t ri = 0; ri < cfg.rounds.size(); ++ri) {
    const RoundConfig& rc = cfg.rounds[ri];
    auto cm = std::make_unique<IrsCommitment<T, T>>(irs_receive<T, T>(rc.irs, vs));
    pow_verify(rc.pow, vs);
    InDomain<T> in_domain = open_prev(ri);
    std::vector<T> pts = cm->ood_points;
    for (auto& p : in_domain.points) pts.push_back(p);
    std::vector<T> vals;
    for (size_t o = 0; o < cm->ood_points.size(); ++o) vals.push_back(cm->ood_matrix[o]);
    std::vector<T> wts = tensor_product(poly_rlc, eq_weights(round_folding.back()));
    size_t cols = in_domain.cols();
    for (size_t pi = 0; pi < in_domain.points.size(); ++pi) {
      std::vector<T> row(in_domain.matrix.begin() + pi * cols, in_domain.matrix.begin() + (pi + 1) * cols);
      vals.push_back(dot(wts, row));
    }
    std::vector<T> rlc = geometric_challenge<T>(vs, vals.size());
    the_sum += dot(rlc, vals);
    constraints.push_back({rlc, pts, rc.irs.vector_size});
    folding = sumcheck_verify<T>(rc.sumcheck, vs, the_sum);
    round_folding.push_back(folding);
    prev = std::move(cm);
  }
  std::vector<T> final_vector;
  for (size_t i = 0; i < cfg.final_sumcheck.initial_size; ++i) final_vector.push_back(recv_elem<T>(vs));
  pow_verify(cfg.final_pow, vs);
  InDomain<T> in_domain = open_prev(cfg.rounds.size());
  {
    std::vector<T> wts = tensor_product(poly_rlc, eq_weights(round_folding.back()));
    size_t cols = in_domain.cols();
    for (size_t pi = 0; pi < in_domain.points.size(); ++pi) {
      std::vector<T> row(in_domain.matrix.begin() + pi * cols, in_domain.matrix.begin() + (pi + 1) * cols);
      T expect = dot(wts, row);
      // UnivariateEvaluation::evaluate of the final vector at the point
      T got = T::zero();
      for (size_t k = final_vector.size(); k-- > 0;) got = got * in_domain.points[pi] + final_vector[k];
      if (got != expect) throw VerificationError();
    }
  }
  std::vector<T> fin = sumcheck_verify<T>(cfg.final_sumcheck, vs, the_sum);
  round_folding.push_back(fin);
  std::vector<T> evaluation_point;
  for (auto& r : round_folding)
    for (auto& x : r) evaluation_point.push_back(x);
  // poly_eval = MLE of the final vector at the final sumcheck randomness
  T poly_eval = T::zero();
  {
    std::vector<T> eq((size_t)1 << fin.size(), T::zero());
    eval_eq(eq, fin, T::one());
    for (size_t i = 0; i < final_vector.size(); ++i) poly_eval += eq[i] * final_vector[i];
  }
  if (poly_eval.is_zero()) throw VerificationError();
  T lf_rlc = the_sum * poly_eval.inv();
  for (size_t r = 0; r < constraints.size(); ++r) {
    size_t num_vars = 0;
    size_t sz = r == 0 ? cfg.initial_size() : cfg.rounds[r - 1].irs.vector_size;
    while (((size_t)1 << num_vars) < sz) ++num_vars;
    (void)initial_num_variables;
    size_t start = evaluation_point.size() >= num_vars ? evaluation_point.size() - num_vars : 0;
    std::vector<T> tail(evaluation_point.begin() + start, evaluation_point.end());
    for (size_t k = 0; k < constraints[r].points.size(); ++k)
      lf_rlc -= constraints[r].rlc[k] * univariate_mle(constraints[r].points[k], tail);
  }
  claim.evaluation_point = evaluation_point;
  claim.rlc_coefficients = init_rlc;
  claim.linear_form_rlc = lf_rlc;
  return claim;
}

template <class T>
bool final_claim_verify(const FinalClaim<T>& c, const LinearForms<T>& forms) {
  if (c.rlc_coefficients.size() != forms.count()) return false;
  T acc = T::zero();
  size_t k = 0;
  for (auto& pt : forms.mle_points) {
    acc += c.rlc_coefficients[k++] * mle_of_eq(pt, c.evaluation_point);
  }
  for (auto& cv : forms.covectors) {
    acc += c.rlc_coefficients[k++] * multilinear_extend<T, T>(cv.data(), cv.size(), c.evaluation_point);
  }
  return acc == c.linear_form_rlc;
}

}  // namespace oracle
