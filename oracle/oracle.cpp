// ORACLE — test infrastructure only. Implementation of the non-template parts of the CPU
// restatement plus the C API the parity tests and the CPU-baseline leg of bench.py load through
// ctypes. The GPU library never links this file.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <sstream>

#include "oracle_api.h"
#include "whir.hpp"

namespace oracle {

// Field192 / Field256 parameters (fields.rs:65-77), little-endian u64 limbs of the modulus.
const MontParams<3>& f192_params() {
  // 3801539170989320091464968600173246866371124347557388484609
  static const uint64_t p[3] = {0x0000000000000001ULL, 0x0000000000000000ULL, 0x0000000000000000ULL};
  static MontParams<3> P = [] {
    // decimal -> limbs at first use
    const char* dec = "3801539170989320091464968600173246866371124347557388484609";
    uint64_t l[3] = {0, 0, 0};
    for (const char* c = dec; *c; ++c) {
      u128 carry = (uint64_t)(*c - '0');
      for (int i = 0; i < 3; ++i) {
        u128 v = (u128)l[i] * 10 + carry;
        l[i] = (uint64_t)v;
        carry = v >> 64;
      }
    }
    return make_mont_params<3>(l, 3, "Field192");
  }();
  (void)p;
  return P;
}
const MontParams<4>& f256_params() {
  static MontParams<4> P = [] {
    const char* dec = "21888242871839275222246405745257275088548364400416034343698204186575808495617";
    uint64_t l[4] = {0, 0, 0, 0};
    for (const char* c = dec; *c; ++c) {
      u128 carry = (uint64_t)(*c - '0');
      for (int i = 0; i < 4; ++i) {
        u128 v = (u128)l[i] * 10 + carry;
        l[i] = (uint64_t)v;
        carry = v >> 64;
      }
    }
    return make_mont_params<4>(l, 5, "Field256");
  }();
  return P;
}

int num_threads() {
  static int n = [] {
    const char* e = getenv("WHIR_ORACLE_THREADS");
    if (e && atoi(e) > 0) return atoi(e);
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
  }();
  return n;
}

void parallel_for(size_t n, size_t min_parallel, const std::function<void(size_t, size_t)>& fn) {
  int T = num_threads();
  if (n == 0) return;
  if (T <= 1 || n < min_parallel || n < 2) {
    fn(0, n);
    return;
  }
  size_t parts = std::min<size_t>((size_t)T, n);
  size_t chunk = (n + parts - 1) / parts;
  std::vector<std::thread> th;
  std::exception_ptr err;
  std::mutex mu;
  for (size_t p = 0; p < parts; ++p) {
    size_t s = p * chunk, e = std::min(n, s + chunk);
    if (s >= e) break;
    th.emplace_back([&, s, e]() {
      try {
        fn(s, e);
      } catch (...) {
        std::lock_guard<std::mutex> g(mu);
        if (!err) err = std::current_exception();
      }
    });
  }
  for (auto& t : th) t.join();
  if (err) std::rethrow_exception(err);
}

// ------------------------------------------------------------------------------------------
// Proof of work: waves of T blocks, the first wave with a hit yields the lowest nonce.
// ------------------------------------------------------------------------------------------
uint64_t pow_grind(HashKind kind, const uint8_t challenge[32], uint64_t threshold) {
  const uint64_t block = 1 << 14;
  int T = num_threads();
  for (uint64_t wave = 0;; ++wave) {
    std::vector<uint64_t> found(T, UINT64_MAX);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) {
      th.emplace_back([&, t]() {
        uint8_t in[64] = {0}, out[32];
        memcpy(in, challenge, 32);
        uint64_t start = (wave * T + t) * block;
        for (uint64_t nonce = start; nonce < start + block; ++nonce) {
          for (int i = 0; i < 8; ++i) in[32 + i] = (uint8_t)(nonce >> (8 * i));
          hash_many(kind, 64, in, 1, out);
          uint64_t v = 0;
          for (int i = 7; i >= 0; --i) v = (v << 8) | out[i];
          if (v <= threshold) {
            found[t] = nonce;
            break;
          }
        }
      });
    }
    for (auto& x : th) x.join();
    uint64_t best = UINT64_MAX;
    for (auto f : found) best = std::min(best, f);
    if (best != UINT64_MAX) return best;
    if (wave > (1ULL << 40)) throw std::runtime_error("Proof of Work failed to solve.");
  }
}

// ------------------------------------------------------------------------------------------
// Merkle tree (merkle_tree.rs:82-273)
// ------------------------------------------------------------------------------------------
std::vector<Digest> merkle_build(const MerkleConfig& c, const std::vector<Digest>& leaves) {
  if (leaves.size() != c.num_leaves) throw std::runtime_error("wrong number of leaf hashes");
  HashKind k = hash_kind(c.hash_id);
  if (k == HK_INVALID) throw std::runtime_error("Hash Engine not found");
  std::vector<Digest> nodes(c.num_nodes());
  memset(nodes.data(), 0, nodes.size() * sizeof(Digest));
  for (size_t i = 0; i < leaves.size(); ++i) nodes[i] = leaves[i];
  size_t prev_off = 0, prev_len = (size_t)1 << c.layers;
  size_t cur_off = prev_len;
  for (size_t layer = 0; layer < c.layers; ++layer) {
    size_t cur_len = prev_len / 2;
    parallel_for(cur_len, 1024, [&](size_t s, size_t e) {
      for (size_t i = s; i < e; ++i) hash_many(k, 64, nodes[prev_off + 2 * i].b, 1, nodes[cur_off + i].b);
    });
    prev_off = cur_off;
    prev_len = cur_len;
    cur_off += cur_len;
  }
  return nodes;
}

std::vector<Digest> merkle_open_hints(const MerkleConfig& c, const std::vector<Digest>& nodes,
                                      const std::vector<size_t>& sorted) {
  std::vector<Digest> hints;
  std::vector<size_t> idx = sorted;
  size_t off = 0, len = (size_t)1 << c.layers;
  while (len > 1) {
    std::vector<size_t> next;
    for (size_t i = 0; i < idx.size(); ++i) {
      size_t a = idx[i];
      if (i + 1 < idx.size() && idx[i + 1] == (a ^ 1)) {
        next.push_back(a >> 1);
        ++i;
      } else {
        hints.push_back(nodes[off + (a ^ 1)]);
        next.push_back(a >> 1);
      }
    }
    idx = next;
    off += len;
    len /= 2;
  }
  return hints;
}

void merkle_verify(const MerkleConfig& c, VerifierState& vs, const Digest& root, const std::vector<size_t>& indices,
                   const std::vector<Digest>& leaf_hashes) {
  if (indices.size() != leaf_hashes.size()) throw VerificationError();
  for (size_t i : indices)
    if (i >= c.num_leaves) throw VerificationError();
  if (indices.empty()) return;
  std::vector<std::pair<size_t, Digest>> layer;
  for (size_t i = 0; i < indices.size(); ++i) layer.push_back({indices[i], leaf_hashes[i]});
  std::stable_sort(layer.begin(), layer.end(), [](auto& a, auto& b) { return a.first < b.first; });
  for (size_t i = 1; i < layer.size(); ++i)
    if (layer[i - 1].first == layer[i].first && layer[i - 1].second != layer[i].second) throw VerificationError();
  std::vector<size_t> idx;
  std::vector<Digest> hs;
  for (size_t i = 0; i < layer.size(); ++i) {
    if (i > 0 && layer[i].first == layer[i - 1].first) continue;
    idx.push_back(layer[i].first);
    hs.push_back(layer[i].second);
  }
  HashKind k = hash_kind(c.hash_id);
  if (k == HK_INVALID) throw VerificationError();
  for (size_t l = 0; l < c.layers; ++l) {
    std::vector<size_t> ni;
    std::vector<Digest> input;
    size_t hp = 0;
    for (size_t i = 0; i < idx.size(); ++i) {
      size_t a = idx[i];
      if (i + 1 < idx.size() && idx[i + 1] == (a ^ 1)) {
        input.push_back(hs[hp++]);
        input.push_back(hs[hp++]);
        ni.push_back(a >> 1);
        ++i;
      } else {
        Digest h;
        vs.hint_bytes(h.b, 32);
        if ((a & 1) == 0) {
          input.push_back(hs[hp++]);
          input.push_back(h);
        } else {
          input.push_back(h);
          input.push_back(hs[hp++]);
        }
        ni.push_back(a >> 1);
      }
    }
    std::vector<Digest> nh(input.size() / 2);
    for (size_t i = 0; i < nh.size(); ++i) hash_many(k, 64, input[2 * i].b, 1, nh[i].b);
    idx = ni;
    hs = nh;
  }
  if (idx.size() != 1 || idx[0] != 0) throw VerificationError();
  if (hs[0] != root) throw VerificationError();
}

// ------------------------------------------------------------------------------------------
// Configuration
// ------------------------------------------------------------------------------------------
IrsConfig irs_config_new(double security_target, bool unique_decoding, const uint8_t hash_id[32], size_t num_vectors,
                         size_t vector_size, size_t interleaving_depth, double rate, double field_bits) {
  if (interleaving_depth == 0 || vector_size % interleaving_depth != 0) throw std::runtime_error("bad interleaving");
  if (!(rate > 0. && rate <= 1.)) throw std::runtime_error("bad rate");
  IrsConfig c;
  size_t message_length = vector_size / interleaving_depth;
  size_t codeword_length = (size_t)std::ceil((double)message_length / rate);
  double r = (double)message_length / (double)codeword_length;
  double js = unique_decoding ? 0.0 : std::sqrt(r) / 20.;
  size_t ood = 0;
  if (!unique_decoding) {
    double list_size = 1. / (2. * js * std::sqrt(r));
    double l_choose_2 = list_size * (list_size - 1.) / 2.;
    double log_per_sample = field_bits - std::log2((double)(vector_size - 1));
    if (!(log_per_sample > 0.)) throw std::runtime_error("field too small for OOD samples");
    double v = std::ceil((security_target + std::log2(l_choose_2)) / log_per_sample);
    ood = (size_t)std::max(v, 1.);
  }
  double per_sample = unique_decoding ? (1. + r) / 2. : std::sqrt(r) + js;
  size_t ids = (size_t)std::ceil(security_target / (-std::log2(per_sample)));
  c.num_vectors = num_vectors;
  c.vector_size = vector_size;
  c.mask_length = 0;
  c.codeword_length = codeword_length;
  c.interleaving_depth = interleaving_depth;
  c.num_cols = interleaving_depth * num_vectors;
  memcpy(c.leaf_hash_id, hash_id, 32);
  c.merkle.num_leaves = codeword_length;
  c.merkle.layers = layers_for_size(codeword_length);
  memcpy(c.merkle.hash_id, hash_id, 32);
  c.johnson_slack = js;
  c.in_domain_samples = ids;
  c.out_domain_samples = ood;
  c.deduplicate_in_domain = false;
  c.field_bits = field_bits;
  return c;
}

static PowConfig make_pow(const uint8_t* hash_id, double bits) {
  PowConfig p;
  memcpy(p.hash_id, hash_id, 32);
  p.threshold = pow_threshold(bits);
  return p;
}

WhirConfig whir_config_new(size_t size, const ProtocolParameters& wp, double field_bits) {
  if (size == 0 || (size & (size - 1))) throw std::runtime_error("Only powers of two size are supported at the moment.");
  WhirConfig cfg;
  double security_level = (double)wp.security_level;
  double protocol_security_level =
      (double)(wp.security_level > wp.pow_bits ? wp.security_level - wp.pow_bits : 0);
  size_t log_inv_rate = wp.starting_log_inv_rate;
  size_t num_variables = 0;
  while (((size_t)1 << num_variables) < size) ++num_variables;
  if (wp.initial_folding_factor > num_variables) throw std::runtime_error("initial folding factor too large");
  cfg.initial_committer =
      irs_config_new(protocol_security_level, wp.unique_decoding, wp.hash_id, wp.batch_size, size,
                     (size_t)1 << wp.initial_folding_factor, std::pow(0.5, (int)wp.starting_log_inv_rate), field_bits);
  const IrsConfig& ic = cfg.initial_committer;
  double starting_folding_pow_bits;
  {
    double prox = ic.rbr_soundness_fold_prox_gaps();
    double log_list = std::log2(ic.list_size());
    double sumcheck_error = field_bits - log_list - 1.;
    double error = std::min(prox, sumcheck_error);
    starting_folding_pow_bits = std::max(security_level - error, 0.);
  }
  double initial_skip_pow_bits;
  {
    double prox = ic.rbr_soundness_fold_prox_gaps() + std::log2((double)wp.initial_folding_factor);
    initial_skip_pow_bits = std::max(security_level - prox, 0.0);
  }
  size_t round = 0;
  size_t in_domain_samples = ic.in_domain_samples;
  double query_error = ic.rbr_queries();
  num_variables -= wp.initial_folding_factor;
  while (num_variables >= wp.folding_factor) {
    size_t rff = round == 0 ? wp.initial_folding_factor : wp.folding_factor;
    size_t next_rate = log_inv_rate + (rff - 1);
    RoundConfig rc;
    rc.irs = irs_config_new(protocol_security_level, wp.unique_decoding, wp.hash_id, 1, (size_t)1 << num_variables,
                            (size_t)1 << wp.folding_factor, std::pow(0.5, (int)next_rate), field_bits);
    double combination_error;
    {
      double log_list = std::log2(rc.irs.list_size());
      size_t count = rc.irs.out_domain_samples + in_domain_samples;
      double log_comb = std::log2((double)count);
      combination_error = field_bits - (log_comb + log_list + 1.);
    }
    double pow_bits = std::max(0., security_level - std::min(query_error, combination_error));
    double folding_pow_bits;
    {
      double prox = rc.irs.rbr_soundness_fold_prox_gaps();
      double log_list = std::log2(rc.irs.list_size());
      double sumcheck_error = field_bits - (log_list + 1.);
      double error = std::min(prox, sumcheck_error);
      folding_pow_bits = std::max(security_level - error, 0.);
    }
    rc.sumcheck.initial_size = (size_t)1 << num_variables;
    rc.sumcheck.round_pow = make_pow(wp.hash_id, folding_pow_bits);
    rc.sumcheck.num_rounds = wp.folding_factor;
    rc.sumcheck.mask_length = 0;
    rc.pow = make_pow(wp.hash_id, pow_bits);
    round += 1;
    num_variables -= wp.folding_factor;
    log_inv_rate = next_rate;
    in_domain_samples = rc.irs.in_domain_samples;
    query_error = rc.irs.rbr_queries();
    cfg.rounds.push_back(rc);
  }
  double rbr_error = cfg.rounds.empty() ? ic.rbr_queries() : cfg.rounds.back().irs.rbr_queries();
  double final_pow_bits = std::max(0., security_level - rbr_error);
  double final_folding_pow_bits = std::max(0., security_level - field_bits + 1.0);
  cfg.initial_sumcheck.initial_size = size;
  cfg.initial_sumcheck.round_pow = make_pow(wp.hash_id, starting_folding_pow_bits);
  cfg.initial_sumcheck.num_rounds = wp.initial_folding_factor;
  cfg.initial_sumcheck.mask_length = 0;
  cfg.initial_skip_pow = make_pow(wp.hash_id, initial_skip_pow_bits);
  cfg.final_sumcheck.initial_size = (size_t)1 << num_variables;
  cfg.final_sumcheck.round_pow = make_pow(wp.hash_id, final_folding_pow_bits);
  cfg.final_sumcheck.num_rounds = num_variables;
  cfg.final_sumcheck.mask_length = 0;
  cfg.final_pow = make_pow(wp.hash_id, final_pow_bits);
  return cfg;
}

// ---- protocol id bytes: ciborium::into_writer(&whir::Config) (transcript/mod.rs:111-121) -------
// The configuration is first built as a tree of serde data-model values (protocols/whir/mod.rs:
// 29-46, irs_commit.rs:51-91, matrix_commit.rs:93-111, merkle_tree.rs:25-40, sumcheck.rs:33-44,
// proof_of_work.rs:23-27, type_info.rs:98-117, fields.rs:32-62, embedding.rs:43-59, 191-205), then
// written as CBOR (RFC 8949) the way ciborium does: shortest heads, definite lengths, floats in the
// shortest IEEE width that holds the value exactly.
namespace {
struct Sv {  // serde value
  enum Kind { UINT, BOOL, FLOAT, BYTES, TEXT, SEQ, STRUCT } kind;
  uint64_t u = 0;
  double f = 0;
  std::string s;                                  // text, or bytes
  std::vector<Sv> items;                          // sequence elements / struct field values
  std::vector<std::string> names;                 // struct field names
  static Sv uint(uint64_t v) { Sv x{UINT}; x.u = v; return x; }
  static Sv boolean(bool v) { Sv x{BOOL}; x.u = v; return x; }
  static Sv real(double v) { Sv x{FLOAT}; x.f = v; return x; }
  static Sv text(const std::string& t) { Sv x{TEXT}; x.s = t; return x; }
  static Sv bytes(const std::vector<uint8_t>& b) { Sv x{BYTES}; x.s.assign(b.begin(), b.end()); return x; }
  static Sv seq(std::vector<Sv> v) { Sv x{SEQ}; x.items = std::move(v); return x; }
  static Sv record(std::vector<std::pair<std::string, Sv>> fields) {
    Sv x{STRUCT};
    for (auto& f : fields) {
      x.names.push_back(f.first);
      x.items.push_back(std::move(f.second));
    }
    return x;
  }
};

void cbor_head(std::vector<uint8_t>& o, int major, uint64_t v) {
  int extra = v < 24 ? 0 : v < (1ull << 8) ? 1 : v < (1ull << 16) ? 2 : v < (1ull << 32) ? 4 : 8;
  int info = extra == 0 ? (int)v : extra == 1 ? 24 : extra == 2 ? 25 : extra == 4 ? 26 : 27;
  o.push_back((uint8_t)((major << 5) | info));
  for (int i = extra - 1; i >= 0; --i) o.push_back((uint8_t)(v >> (8 * i)));
}

// IEEE binary16 bit pattern of v if it holds v exactly.
bool half_exact(double v, uint16_t& out) {
  uint64_t b;
  memcpy(&b, &v, 8);
  const uint64_t sign = b >> 63;
  const int exp = (int)((b >> 52) & 0x7ff);
  const uint64_t man = b & ((1ull << 52) - 1);
  if (exp == 0x7ff) return false;  // not produced by the configuration
  if (exp == 0 && man == 0) {
    out = (uint16_t)(sign << 15);
    return true;
  }
  if (exp == 0) return false;  // binary64 subnormals are far below binary16's range
  const int e = exp - 1023;  // v = 1.man * 2^e
  if (e >= -14 && e <= 15) {
    if (man & ((1ull << 42) - 1)) return false;  // more than 10 mantissa bits
    out = (uint16_t)((sign << 15) | ((uint64_t)(e + 15) << 10) | (man >> 42));
    return true;
  }
  if (e >= -24 && e < -14) {  // binary16 subnormal: v = k * 2^-24
    const uint64_t full = man | (1ull << 52);
    const int shift = 52 - (e + 24);  // k = full >> shift
    if (full & ((1ull << shift) - 1)) return false;
    out = (uint16_t)((sign << 15) | (full >> shift));
    return true;
  }
  return false;
}

void cbor_write(std::vector<uint8_t>& o, const Sv& v) {
  switch (v.kind) {
    case Sv::UINT: cbor_head(o, 0, v.u); break;
    case Sv::BOOL: o.push_back(v.u ? 0xf5 : 0xf4); break;
    case Sv::BYTES:
    case Sv::TEXT:
      cbor_head(o, v.kind == Sv::BYTES ? 2 : 3, v.s.size());
      o.insert(o.end(), v.s.begin(), v.s.end());
      break;
    case Sv::SEQ:
      cbor_head(o, 4, v.items.size());
      for (const Sv& x : v.items) cbor_write(o, x);
      break;
    case Sv::STRUCT:
      cbor_head(o, 5, v.items.size());
      for (size_t i = 0; i < v.items.size(); ++i) {
        cbor_write(o, Sv::text(v.names[i]));
        cbor_write(o, v.items[i]);
      }
      break;
    case Sv::FLOAT: {
      uint16_t h;
      const float f = (float)v.f;
      if (half_exact(v.f, h)) {
        o.push_back(0xf9);
        o.push_back((uint8_t)(h >> 8));
        o.push_back((uint8_t)h);
      } else if ((double)f == v.f) {
        uint32_t b;
        memcpy(&b, &f, 4);
        o.push_back(0xfa);
        for (int i = 3; i >= 0; --i) o.push_back((uint8_t)(b >> (8 * i)));
      } else {
        uint64_t b;
        memcpy(&b, &v.f, 8);
        o.push_back(0xfb);
        for (int i = 7; i >= 0; --i) o.push_back((uint8_t)(b >> (8 * i)));
      }
      break;
    }
  }
}

Sv engine_sv(const uint8_t* id) {
  std::vector<Sv> v;
  for (int i = 0; i < 32; ++i) v.push_back(Sv::uint(id[i]));
  return Sv::seq(std::move(v));
}
// FieldInfo of a field whose characteristic is the oracle's field `kind` base prime.
Sv field_info_sv(int kind, uint64_t degree) {
  std::vector<uint64_t> limbs;
  if (kind == ORACLE_FIELD192) {
    limbs.assign(f192_params().p, f192_params().p + 3);
  } else if (kind == ORACLE_FIELD256) {
    limbs.assign(f256_params().p, f256_params().p + 4);
  } else {
    limbs.push_back(GL_P);
  }
  std::vector<uint8_t> be;
  for (size_t i = limbs.size(); i-- > 0;)
    for (int b = 7; b >= 0; --b) be.push_back((uint8_t)(limbs[i] >> (8 * b)));
  size_t lead = 0;
  while (lead < be.size() && be[lead] == 0) ++lead;
  be.erase(be.begin(), be.begin() + lead);
  return Sv::record({{"characteristic", Sv::bytes(be)}, {"extension_degree", Sv::uint(degree)}});
}
uint64_t target_degree(int kind) { return kind == ORACLE_GOLDILOCKS2 ? 2 : kind == ORACLE_GOLDILOCKS3 ? 3 : 1; }

Sv pow_sv(const PowConfig& p) {
  return Sv::record({{"hash_id", engine_sv(p.hash_id)}, {"threshold", Sv::uint(p.threshold)}});
}
Sv sumcheck_sv(const SumcheckConfig& s, int kind) {
  return Sv::record({{"field", field_info_sv(kind, target_degree(kind))},
                     {"initial_size", Sv::uint(s.initial_size)},
                     {"round_pow", pow_sv(s.round_pow)},
                     {"num_rounds", Sv::uint(s.num_rounds)},
                     {"mask_length", Sv::uint(s.mask_length)}});
}
// identity = true: irs_commit::Config<Identity<Target>>; else the config's own embedding.
Sv irs_sv(const IrsConfig& c, int kind, bool identity) {
  const uint64_t deg = target_degree(kind);
  const bool base = !identity && deg > 1;
  Sv emb = Sv::record({{"type", Sv::text(base ? "basefield" : "identity")},
                       {"value", Sv::record({{base ? "extension" : "field", field_info_sv(kind, deg)}})}});
  std::vector<Sv> layers;
  for (size_t l = 0; l < c.merkle.layers; ++l) layers.push_back(Sv::record({{"hash_id", engine_sv(c.merkle.hash_id)}}));
  Sv merkle = Sv::record({{"num_leaves", Sv::uint(c.merkle.num_leaves)}, {"layers", Sv::seq(std::move(layers))}});
  Sv matrix = Sv::record({{"element_type", field_info_sv(kind, base ? 1 : deg)},
                          {"num_cols", Sv::uint(c.num_cols)},
                          {"leaf_hash_id", engine_sv(c.leaf_hash_id)},
                          {"merkle_tree", std::move(merkle)}});
  return Sv::record({{"embedding", std::move(emb)},
                     {"num_vectors", Sv::uint(c.num_vectors)},
                     {"vector_size", Sv::uint(c.vector_size)},
                     {"mask_length", Sv::uint(c.mask_length)},
                     {"codeword_length", Sv::uint(c.codeword_length)},
                     {"interleaving_depth", Sv::uint(c.interleaving_depth)},
                     {"matrix_commit", std::move(matrix)},
                     {"johnson_slack", Sv::real(c.johnson_slack)},
                     {"in_domain_samples", Sv::uint(c.in_domain_samples)},
                     {"out_domain_samples", Sv::uint(c.out_domain_samples)},
                     {"deduplicate_in_domain", Sv::boolean(c.deduplicate_in_domain)}});
}
}  // namespace

std::vector<uint8_t> config_bytes(const WhirConfig& c, int field_kind) {
  std::vector<Sv> rounds;
  for (const auto& r : c.rounds)
    rounds.push_back(Sv::record({{"irs_committer", irs_sv(r.irs, field_kind, true)},
                                 {"sumcheck", sumcheck_sv(r.sumcheck, field_kind)},
                                 {"pow", pow_sv(r.pow)}}));
  Sv cfg = Sv::record({{"initial_committer", irs_sv(c.initial_committer, field_kind, false)},
                       {"initial_sumcheck", sumcheck_sv(c.initial_sumcheck, field_kind)},
                       {"initial_skip_pow", pow_sv(c.initial_skip_pow)},
                       {"round_configs", Sv::seq(std::move(rounds))},
                       {"final_sumcheck", sumcheck_sv(c.final_sumcheck, field_kind)},
                       {"final_pow", pow_sv(c.final_pow)}});
  std::vector<uint8_t> o;
  cbor_write(o, cfg);
  return o;
}

static void json_irs(std::ostringstream& s, const IrsConfig& c) {
  s << "{\"num_vectors\":" << c.num_vectors << ",\"vector_size\":" << c.vector_size
    << ",\"codeword_length\":" << c.codeword_length << ",\"interleaving_depth\":" << c.interleaving_depth
    << ",\"num_cols\":" << c.num_cols << ",\"merkle_layers\":" << c.merkle.layers
    << ",\"in_domain_samples\":" << c.in_domain_samples << ",\"out_domain_samples\":" << c.out_domain_samples
    << ",\"johnson_slack\":" << c.johnson_slack << "}";
}
static void json_sc(std::ostringstream& s, const SumcheckConfig& c) {
  s << "{\"initial_size\":" << c.initial_size << ",\"num_rounds\":" << c.num_rounds
    << ",\"round_pow_threshold\":" << c.round_pow.threshold << "}";
}
std::string config_json(const WhirConfig& c) {
  std::ostringstream s;
  s.precision(17);
  s << "{\"initial_committer\":";
  json_irs(s, c.initial_committer);
  s << ",\"initial_sumcheck\":";
  json_sc(s, c.initial_sumcheck);
  s << ",\"initial_skip_pow_threshold\":" << c.initial_skip_pow.threshold << ",\"rounds\":[";
  for (size_t i = 0; i < c.rounds.size(); ++i) {
    if (i) s << ",";
    s << "{\"irs\":";
    json_irs(s, c.rounds[i].irs);
    s << ",\"sumcheck\":";
    json_sc(s, c.rounds[i].sumcheck);
    s << ",\"pow_threshold\":" << c.rounds[i].pow.threshold << "}";
  }
  s << "],\"final_sumcheck\":";
  json_sc(s, c.final_sumcheck);
  s << ",\"final_pow_threshold\":" << c.final_pow.threshold << "}";
  return s.str();
}

}  // namespace oracle

// =============================================================================================
// C API
// =============================================================================================
using namespace oracle;

namespace {
thread_local std::string g_err;
int fail(const char* msg) {
  g_err = msg;
  return -1;
}

template <class Fn>
int guard(Fn fn) {
  try {
    return fn();
  } catch (const VerificationError&) {
    g_err = "verification failed";
    return 1;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Dispatch on the embedding id: calls f.template operator()<S, T>().
template <class Fn>
int with_embedding(int field, Fn&& f) {
  switch (field) {
    case ORACLE_GOLDILOCKS1: return f.template operator()<Gl, Gl>();
    case ORACLE_GOLDILOCKS2: return f.template operator()<Gl, Gl2>();
    case ORACLE_GOLDILOCKS3: return f.template operator()<Gl, Gl3>();
    case ORACLE_FIELD192: return f.template operator()<F192, F192>();
    case ORACLE_FIELD256: return f.template operator()<F256, F256>();
    default: return fail("unknown field id");
  }
}
// Dispatch on a single field type (target of the embedding for ext ids).
template <class Fn>
int with_field(int field, Fn&& f) {
  switch (field) {
    case ORACLE_GOLDILOCKS1: return f.template operator()<Gl>();
    case ORACLE_GOLDILOCKS2: return f.template operator()<Gl2>();
    case ORACLE_GOLDILOCKS3: return f.template operator()<Gl3>();
    case ORACLE_FIELD192: return f.template operator()<F192>();
    case ORACLE_FIELD256: return f.template operator()<F256>();
    default: return fail("unknown field id");
  }
}

template <class F>
std::vector<F> load(const uint64_t* p, size_t n) {
  std::vector<F> v(n);
  constexpr int L = elem_limbs<F>();
  for (size_t i = 0; i < n; ++i) {
    if (!elem_limbs_valid<F>(p + i * L)) throw std::runtime_error("non-canonical field element");
    v[i] = elem_from_limbs<F>(p + i * L);
  }
  return v;
}
template <class F>
void store(const std::vector<F>& v, uint64_t* p) {
  constexpr int L = elem_limbs<F>();
  for (size_t i = 0; i < v.size(); ++i) elem_to_limbs<F>(v[i], p + i * L);
}

ProtocolParameters to_params(const oracle_protocol_params* p) {
  ProtocolParameters w;
  w.unique_decoding = p->unique_decoding != 0;
  w.starting_log_inv_rate = p->starting_log_inv_rate;
  w.initial_folding_factor = p->initial_folding_factor;
  w.folding_factor = p->folding_factor;
  w.security_level = p->security_level;
  w.pow_bits = p->pow_bits;
  w.batch_size = p->batch_size;
  memcpy(w.hash_id, p->hash_id, 32);
  return w;
}
}  // namespace

struct oracle_proof {
  std::vector<uint8_t> narg, hints;
  std::vector<uint64_t> eval_point, rlc;
  std::vector<uint8_t> roots;  // commitment roots (32 bytes each) in transcript order
  std::string config;
};

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }
int oracle_num_threads(void) { return num_threads(); }

int oracle_field_limbs(int field) {
  return with_field(field, []<class F>() { return elem_limbs<F>(); });
}

int oracle_field_op(int field, int op, const uint64_t* a, const uint64_t* b, uint64_t* out, size_t n) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      constexpr int L = elem_limbs<F>();
      for (size_t i = 0; i < n; ++i) {
        F x = elem_from_limbs<F>(a + i * L), y = b ? elem_from_limbs<F>(b + i * L) : F::zero(), r;
        switch (op) {
          case 0: r = x + y; break;
          case 1: r = x - y; break;
          case 2: r = x * y; break;
          case 3: r = x.inv(); break;
          case 4: r = -x; break;
          default: throw std::runtime_error("bad op");
        }
        elem_to_limbs<F>(r, out + i * L);
      }
      return 0;
    });
  });
}

int oracle_ntt_root(int field, uint64_t order, uint64_t* out) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      F r = F::from_base(prime_root<typename F::Base>(order));
      elem_to_limbs<F>(r, out);
      return 0;
    });
  });
}

int oracle_next_order(int field, uint64_t size, uint64_t* out) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      if (!next_order<typename F::Base>(size, out)) return fail("size exceeds largest supported order");
      return 0;
    });
  });
}

int oracle_interleaved_encode(int field, const uint64_t* msgs, size_t n_msgs, size_t msg_len, const uint64_t* masks,
                              size_t mask_len, size_t codeword_len, uint64_t* out) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      std::vector<F> m = load<F>(msgs, n_msgs * msg_len);
      std::vector<F> mk = load<F>(masks, n_msgs * mask_len);
      std::vector<const F*> ptrs;
      for (size_t i = 0; i < n_msgs; ++i) ptrs.push_back(m.data() + i * msg_len);
      std::vector<F> cw = interleaved_encode<F>(ptrs, msg_len, mk.data(), mask_len, codeword_len);
      store<F>(cw, out);
      return 0;
    });
  });
}

int oracle_evaluation_points(int field, size_t masked_len, size_t codeword_len, const uint64_t* idx, size_t n,
                             uint64_t* out) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      std::vector<size_t> ix(idx, idx + n);
      auto pts = evaluation_points<typename F::Base>(masked_len, codeword_len, ix);
      std::vector<F> lifted;
      for (auto& p : pts) lifted.push_back(F::from_base(p));
      store<F>(lifted, out);
      return 0;
    });
  });
}

int oracle_hash_many(const uint8_t* engine_id, size_t size, const uint8_t* in, size_t count, uint8_t* out) {
  HashKind k = hash_kind(engine_id);
  if (k == HK_INVALID) return fail("unknown hash engine");
  if (hash_many(k, size, in, count, out)) return fail("unsupported message size");
  return 0;
}

int oracle_sha3_512(const uint8_t* in, size_t n, uint8_t* out) {
  sha3_512(in, n, out);
  return 0;
}

int oracle_merkle_commit(const uint8_t* engine_id, const uint8_t* leaves, size_t n_leaves, uint8_t* nodes_out,
                         size_t* num_nodes) {
  return guard([&] {
    MerkleConfig c;
    c.num_leaves = n_leaves;
    c.layers = layers_for_size(n_leaves);
    memcpy(c.hash_id, engine_id, 32);
    if (num_nodes) *num_nodes = c.num_nodes();
    if (!nodes_out) return 0;
    std::vector<Digest> lv(n_leaves);
    memcpy(lv.data(), leaves, n_leaves * 32);
    auto nodes = merkle_build(c, lv);
    memcpy(nodes_out, nodes.data(), nodes.size() * 32);
    return 0;
  });
}

int oracle_layers_for_size(size_t n) { return (int)layers_for_size(n); }

int oracle_hash_rows(int field, const uint8_t* engine_id, const uint64_t* matrix, size_t rows, size_t cols,
                     uint8_t* out) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      HashKind k = hash_kind(engine_id);
      if (k == HK_INVALID) return fail("unknown hash engine");
      std::vector<F> m = load<F>(matrix, rows * cols);
      auto d = hash_rows<F>(k, m.data(), rows, cols);
      memcpy(out, d.data(), rows * 32);
      return 0;
    });
  });
}

int oracle_sumcheck_poly(int field, const uint64_t* a, size_t na, const uint64_t* b, size_t nb, uint64_t* c0,
                         uint64_t* c2) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      auto va = load<F>(a, na), vb = load<F>(b, nb);
      F x0, x2;
      compute_sumcheck_polynomial(va, vb, &x0, &x2);
      elem_to_limbs<F>(x0, c0);
      elem_to_limbs<F>(x2, c2);
      return 0;
    });
  });
}

int oracle_fold(int field, uint64_t* v, size_t n, const uint64_t* w, size_t* new_len) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      auto vv = load<F>(v, n);
      F ww = elem_from_limbs<F>(w);
      fold(vv, ww);
      store<F>(vv, v);
      *new_len = vv.size();
      return 0;
    });
  });
}

int oracle_eval_eq(int field, uint64_t* acc, const uint64_t* point, size_t nvars, const uint64_t* scalar) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      auto va = load<F>(acc, (size_t)1 << nvars);
      auto pt = load<F>(point, nvars);
      eval_eq(va, pt, elem_from_limbs<F>(scalar));
      store<F>(va, acc);
      return 0;
    });
  });
}

int oracle_geometric_accumulate(int field, uint64_t* acc, size_t n, const uint64_t* scalars, const uint64_t* points,
                                size_t m) {
  return guard([&] {
    return with_field(field, [&]<class F>() {
      auto va = load<F>(acc, n);
      auto s = load<F>(scalars, m), p = load<F>(points, m);
      geometric_accumulate(va, s, p);
      store<F>(va, acc);
      return 0;
    });
  });
}

// Horner of `n` base-field coefficients at a target-field point (embedding id selects both).
int oracle_univariate_evaluate(int field, const uint64_t* coeffs, size_t n, const uint64_t* point, uint64_t* out) {
  return guard([&] {
    return with_embedding(field, [&]<class S, class T>() {
      auto c = load<S>(coeffs, n);
      T x = elem_from_limbs<T>(point);
      T r = univariate_evaluate<T, S>(c.data(), n, x);
      elem_to_limbs<T>(r, out);
      return 0;
    });
  });
}

int oracle_multilinear_extend(int field, const uint64_t* evals, size_t n, const uint64_t* point, size_t nvars,
                              uint64_t* out) {
  return guard([&] {
    return with_embedding(field, [&]<class S, class T>() {
      auto e = load<S>(evals, n);
      auto pt = load<T>(point, nvars);
      T r = multilinear_extend<T, S>(e.data(), n, pt);
      elem_to_limbs<T>(r, out);
      return 0;
    });
  });
}

int oracle_pow_threshold(double bits, uint64_t* out) {
  return guard([&] {
    *out = pow_threshold(bits);
    return 0;
  });
}
double oracle_pow_difficulty(uint64_t threshold) { return pow_difficulty(threshold); }

int oracle_pow_grind(const uint8_t* engine_id, const uint8_t* challenge, uint64_t threshold, uint64_t* nonce) {
  return guard([&] {
    HashKind k = hash_kind(engine_id);
    if (k == HK_INVALID) return fail("unknown hash engine");
    *nonce = pow_grind(k, challenge, threshold);
    return 0;
  });
}

// Replays fixed "squeezed" bytes into challenge_indices (the reference's MockSponge tests).
struct ByteReplay {
  const uint8_t* b;
  size_t n, pos = 0;
  void verifier_bytes(uint8_t* out, size_t k) {
    if (n - pos < k) throw std::runtime_error("replay exhausted");
    memcpy(out, b + pos, k);
    pos += k;
  }
};
int oracle_challenge_indices_replay(const uint8_t* bytes, size_t nbytes, size_t num_leaves, size_t count, int dedup,
                                    uint64_t* out, size_t* out_len) {
  return guard([&] {
    ByteReplay r{bytes, nbytes};
    auto v = challenge_indices(r, num_leaves, count, dedup != 0);
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
    *out_len = v.size();
    return 0;
  });
}

int oracle_sponge_squeeze(const uint8_t* absorb, size_t n_absorb, uint8_t* out, size_t n_out) {
  DuplexSponge s;
  s.absorb(absorb, n_absorb);
  s.squeeze(out, n_out);
  return 0;
}

static int config_for(int field, const oracle_protocol_params* p, size_t num_variables, WhirConfig* out) {
  return with_field(field, [&]<class F>() {
    *out = whir_config_new((size_t)1 << num_variables, to_params(p), field_size_bits<F>());
    return 0;
  });
}

int oracle_whir_config_json(int field, const oracle_protocol_params* p, size_t num_variables, char* out, size_t cap) {
  return guard([&] {
    WhirConfig c;
    if (config_for(field, p, num_variables, &c)) return -1;
    std::string j = config_json(c);
    if (j.size() + 1 > cap) return fail("buffer too small");
    memcpy(out, j.c_str(), j.size() + 1);
    return 0;
  });
}

int oracle_whir_config_bytes(int field, const oracle_protocol_params* p, size_t num_variables, uint8_t* out,
                             size_t cap, size_t* len) {
  return guard([&] {
    WhirConfig c;
    if (config_for(field, p, num_variables, &c)) return -1;
    auto b = config_bytes(c, field);
    *len = b.size();
    if (out) {
      if (b.size() > cap) return fail("buffer too small");
      memcpy(out, b.data(), b.size());
    }
    return 0;
  });
}

double oracle_field_size_bits(int field) {
  double r = 0;
  with_field(field, [&]<class F>() {
    r = field_size_bits<F>();
    return 0;
  });
  return r;
}

int oracle_whir_prove(int field, const oracle_protocol_params* p, size_t num_variables, const char* session,
                      size_t n_witnesses, const uint64_t* vectors, size_t n_points, const uint64_t* points,
                      size_t n_covectors, const uint64_t* covectors, const uint64_t* evaluations,
                      oracle_proof** out) {
  return guard([&] {
    return with_embedding(field, [&]<class S, class T>() {
      WhirConfig cfg = whir_config_new((size_t)1 << num_variables, to_params(p), field_size_bits<T>());
      size_t n = (size_t)1 << num_variables;
      size_t bs = cfg.initial_committer.num_vectors;
      size_t nv = n_witnesses * bs;
      auto vecs = load<S>(vectors, nv * n);
      LinearForms<T> forms;
      for (size_t i = 0; i < n_points; ++i) forms.mle_points.push_back(load<T>(points + i * num_variables * elem_limbs<T>(), num_variables));
      for (size_t i = 0; i < n_covectors; ++i) forms.covectors.push_back(load<T>(covectors + i * n * elem_limbs<T>(), n));
      auto evals = load<T>(evaluations, forms.count() * nv);
      DomainSeparator ds = DomainSeparator::make(config_bytes(cfg, field), session ? session : "");
      ProverState ps(ds);
      auto* res = new oracle_proof();
      std::vector<std::unique_ptr<IrsWitness<S, T>>> ws;
      std::vector<const S*> vptr;
      for (size_t w = 0; w < n_witnesses; ++w) {
        std::vector<const S*> mine;
        for (size_t k = 0; k < bs; ++k) mine.push_back(vecs.data() + (w * bs + k) * n);
        ws.push_back(std::make_unique<IrsWitness<S, T>>(irs_commit<S, T>(cfg.initial_committer, ps, mine)));
        res->roots.insert(res->roots.end(), ws.back()->nodes.back().b, ws.back()->nodes.back().b + 32);
        for (auto* v : mine) vptr.push_back(v);
      }
      std::vector<const IrsWitness<S, T>*> wp;
      for (auto& w : ws) wp.push_back(w.get());
      FinalClaim<T> claim = whir_prove<S, T>(cfg, ps, vptr, wp, forms, evals);
      res->narg = ps.narg;
      res->hints = ps.hints;
      res->eval_point.resize(claim.evaluation_point.size() * elem_limbs<T>());
      store<T>(claim.evaluation_point, res->eval_point.data());
      res->rlc.resize(claim.rlc_coefficients.size() * elem_limbs<T>());
      store<T>(claim.rlc_coefficients, res->rlc.data());
      res->config = config_json(cfg);
      *out = res;
      return 0;
    });
  });
}

size_t oracle_proof_narg(const oracle_proof* p, const uint8_t** data) {
  *data = p->narg.data();
  return p->narg.size();
}
size_t oracle_proof_hints(const oracle_proof* p, const uint8_t** data) {
  *data = p->hints.data();
  return p->hints.size();
}
size_t oracle_proof_eval_point(const oracle_proof* p, const uint64_t** data) {
  *data = p->eval_point.data();
  return p->eval_point.size();
}
size_t oracle_proof_rlc(const oracle_proof* p, const uint64_t** data) {
  *data = p->rlc.data();
  return p->rlc.size();
}
size_t oracle_proof_roots(const oracle_proof* p, const uint8_t** data) {
  *data = p->roots.data();
  return p->roots.size();
}
void oracle_proof_free(oracle_proof* p) { delete p; }

int oracle_whir_verify(int field, const oracle_protocol_params* p, size_t num_variables, const char* session,
                       size_t n_commitments, size_t n_points, const uint64_t* points, size_t n_covectors,
                       const uint64_t* covectors, const uint64_t* evaluations, const uint8_t* narg, size_t narg_len,
                       const uint8_t* hints, size_t hints_len) {
  return guard([&] {
    return with_embedding(field, [&]<class S, class T>() {
      WhirConfig cfg = whir_config_new((size_t)1 << num_variables, to_params(p), field_size_bits<T>());
      size_t n = (size_t)1 << num_variables;
      size_t nv = n_commitments * cfg.initial_committer.num_vectors;
      LinearForms<T> forms;
      for (size_t i = 0; i < n_points; ++i) forms.mle_points.push_back(load<T>(points + i * num_variables * elem_limbs<T>(), num_variables));
      for (size_t i = 0; i < n_covectors; ++i) forms.covectors.push_back(load<T>(covectors + i * n * elem_limbs<T>(), n));
      auto evals = load<T>(evaluations, forms.count() * nv);
      DomainSeparator ds = DomainSeparator::make(config_bytes(cfg, field), session ? session : "");
      VerifierState vs(ds, narg, narg_len, hints, hints_len);
      std::vector<std::unique_ptr<IrsCommitment<S, T>>> cms;
      for (size_t c = 0; c < n_commitments; ++c)
        cms.push_back(std::make_unique<IrsCommitment<S, T>>(irs_receive<S, T>(cfg.initial_committer, vs)));
      std::vector<const IrsCommitment<S, T>*> cp;
      for (auto& c : cms) cp.push_back(c.get());
      FinalClaim<T> claim = whir_verify<S, T>(cfg, vs, cp, evals, num_variables);
      if (!vs.eof()) throw VerificationError();
      if (!final_claim_verify(claim, forms)) throw VerificationError();
      return 0;
    });
  });
}

}  // extern "C"
