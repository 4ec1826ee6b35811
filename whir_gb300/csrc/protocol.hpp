// Host-side protocol logic of the GB300 WHIR prover: parameter selection, Fiat–Shamir transcript,
// element codecs, query sampling and Merkle opening bookkeeping. Only O(queries) work lives here;
// everything proportional to the polynomial size runs in the CUDA kernels.
//
// Parameter selection restates whir::Config::new (src/protocols/whir/config.rs:16-152) and
// irs_commit::Config::new / rbr_* (src/protocols/irs_commit.rs:125-288, 585-630) with the same f64
// expressions; the host compiler runs with -ffp-contract=off so no fused multiply-add changes a
// rounding. The transcript has the reference's interaction structure (src/transcript/mod.rs) on a
// Keccak-f[1600] duplex sponge of this library (the reference's spongefish sponge is not
// available); its exact byte rules are documented in sponge.cuh.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "field.cuh"
#include "hash.cuh"
#include "sponge.cuh"

namespace whir {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------------------------------------
// Engines
// ---------------------------------------------------------------------------------------------
static const uint8_t ENGINE_IDS[5][32] = {
    {0x03, 0xe0, 0x17, 0x49, 0xeb, 0xcc, 0x04, 0x77, 0x92, 0x42, 0x54, 0xeb, 0x48, 0x20, 0x66, 0xb8,
     0x64, 0xa8, 0xdd, 0x4d, 0x77, 0x25, 0x24, 0x64, 0xca, 0x6f, 0x5b, 0x6f, 0x5c, 0xc0, 0x5b, 0x4c},  // Blake3
    {0x01, 0x8e, 0xaa, 0x24, 0x7c, 0xb8, 0x95, 0x7a, 0xb1, 0xe9, 0xfd, 0xac, 0x88, 0x54, 0x50, 0x40,
     0x3c, 0x5e, 0x7b, 0xda, 0x1a, 0xca, 0xaa, 0x50, 0x4e, 0x4c, 0xc8, 0xf2, 0xf7, 0x6b, 0xb0, 0x76},  // SHA2
    {0xaa, 0x80, 0x2d, 0xcd, 0xab, 0xad, 0x8e, 0xa8, 0xa1, 0x43, 0x09, 0x19, 0x89, 0x3b, 0x96, 0xc3,
     0x0e, 0x31, 0xff, 0x57, 0x34, 0xb3, 0x85, 0x99, 0x91, 0x08, 0xaa, 0x20, 0x2d, 0x27, 0xdc, 0x12},  // SHA3
    {0xdd, 0xd2, 0x48, 0x96, 0x4e, 0x32, 0x03, 0x12, 0xa6, 0x67, 0x75, 0xae, 0xe8, 0xe1, 0x6c, 0x88,
     0xc9, 0x27, 0x73, 0x4b, 0xe5, 0x9a, 0xca, 0x09, 0xb7, 0xaf, 0x6d, 0xeb, 0x0a, 0xd0, 0x0e, 0x8c},  // Keccak
    {0x09, 0x45, 0x90, 0x20, 0xf4, 0x51, 0x87, 0x4a, 0x1b, 0x39, 0x98, 0x19, 0xd0, 0x79, 0x63, 0x2c,
     0xc0, 0xf9, 0x26, 0x3b, 0x14, 0x86, 0xc4, 0x23, 0x17, 0x3c, 0x6e, 0x15, 0xd8, 0xe2, 0xd6, 0x1d}};  // Copy

inline int engine_kind(const uint8_t id[32]) {
  for (int k = 0; k < 5; ++k)
    if (!memcmp(id, ENGINE_IDS[k], 32)) return k;
  return -1;
}

// Host hashing of one message (transcript domain separation, verifier-side checks, small inputs).
inline void host_hash(int kind, const uint8_t* msg, size_t len, uint8_t out[32]);

// ---------------------------------------------------------------------------------------------
// Keccak-based helpers on the host
// ---------------------------------------------------------------------------------------------
inline void keccak_hash(const uint8_t* in, size_t len, size_t rate, uint8_t pad, uint8_t* out, size_t outlen) {
  uint64_t st[25] = {0};
  uint8_t* sb = reinterpret_cast<uint8_t*>(st);
  size_t off = 0;
  while (len - off >= rate) {
    for (size_t i = 0; i < rate; ++i) sb[i] ^= in[off + i];
    keccak_f1600(st);
    off += rate;
  }
  for (size_t i = 0; i < len - off; ++i) sb[i] ^= in[off + i];
  sb[len - off] ^= pad;
  sb[rate - 1] ^= 0x80;
  keccak_f1600(st);
  size_t done = 0;
  while (done < outlen) {
    size_t n = std::min(rate, outlen - done);
    memcpy(out + done, sb, n);
    done += n;
    if (done < outlen) keccak_f1600(st);
  }
}
inline void sha3_256_host(const uint8_t* in, size_t len, uint8_t out[32]) { keccak_hash(in, len, 136, 0x06, out, 32); }
inline void sha3_512_host(const uint8_t* in, size_t len, uint8_t out[64]) { keccak_hash(in, len, 72, 0x06, out, 64); }

inline void host_hash(int kind, const uint8_t* msg, size_t len, uint8_t out[32]) {
  if (kind == HASH_COPY) {
    memset(out, 0, 32);
    memcpy(out, msg, std::min<size_t>(len, 32));
    return;
  }
  if (kind == HASH_SHA3) return keccak_hash(msg, len, 136, 0x06, out, 32);
  if (kind == HASH_KECCAK) return keccak_hash(msg, len, 136, 0x01, out, 32);
  // BLAKE3 / SHA-256 on word-aligned messages through the shared word hashers.
  if (len % 4 != 0 || (kind == HASH_BLAKE3 && len > 1024)) throw Error(-2, "host hash: unsupported message size");
  uint32_t o[8];
  auto run = [&](auto& h) {
    h.init((uint32_t)len);
    for (size_t k = 0; k < len; k += 4)
      h.push((uint32_t)msg[k] | ((uint32_t)msg[k + 1] << 8) | ((uint32_t)msg[k + 2] << 16) | ((uint32_t)msg[k + 3] << 24));
    h.finish(o);
  };
  if (kind == HASH_BLAKE3) {
    WordHasher<HASH_BLAKE3> h;
    run(h);
  } else {
    WordHasher<HASH_SHA2> h;
    run(h);
  }
  for (int i = 0; i < 8; ++i)
    for (int b = 0; b < 4; ++b) out[4 * i + b] = (uint8_t)(o[i] >> (8 * b));
}

// ---------------------------------------------------------------------------------------------
// Transcript (the sponge and its byte rules are in sponge.cuh)
// ---------------------------------------------------------------------------------------------
// ProverState: NARG string (prover messages, absorbed) plus out-of-band hints (not absorbed).
struct Transcript {
  Sponge sponge;
  std::vector<uint8_t> narg, hints;
  Transcript() { sponge.reset(); }
  void init(const uint8_t protocol_id[64], const uint8_t session_id[32]) {
    sponge.reset();
    narg.clear();
    hints.clear();
    sponge.absorb(protocol_id, 64);
    sponge.absorb(session_id, 32);
  }
  void prover_bytes(const uint8_t* b, size_t n) {
    narg.insert(narg.end(), b, b + n);
    sponge.absorb(b, n);
  }
  void verifier_bytes(uint8_t* out, size_t n) { sponge.squeeze(out, n); }
  void hint_bytes(const uint8_t* b, size_t n) { hints.insert(hints.end(), b, b + n); }
};

inline std::vector<uint8_t> cbor_text(const std::string& s) {
  std::vector<uint8_t> out;
  size_t n = s.size();
  if (n < 24) {
    out.push_back((uint8_t)(0x60 | n));
  } else if (n < 256) {
    out.push_back(0x78);
    out.push_back((uint8_t)n);
  } else if (n < 65536) {
    out.push_back(0x79);
    out.push_back((uint8_t)(n >> 8));
    out.push_back((uint8_t)n);
  } else {
    out.push_back(0x7a);
    for (int i = 3; i >= 0; --i) out.push_back((uint8_t)(n >> (8 * i)));
  }
  out.insert(out.end(), s.begin(), s.end());
  return out;
}

// ---------------------------------------------------------------------------------------------
// Element codecs on the transcript (byte rules in sponge.cuh)
// ---------------------------------------------------------------------------------------------
template <class F>
inline void send_elem(Transcript& t, const F& x) {
  uint8_t b[8 * F::LIMBS];
  elem_bytes(x, b);
  t.prover_bytes(b, sizeof(b));
}
// Raw in-memory words of an element (host-internal storage, not an encoding).
template <class F>
inline void put_raw(std::vector<uint64_t>& dst, const F& x) {
  const uint64_t* w = reinterpret_cast<const uint64_t*>(&x);
  dst.insert(dst.end(), w, w + F::LIMBS);
}
template <class F>
inline F get_raw(const uint64_t* w) {
  F x;
  memcpy(&x, w, sizeof(F));
  return x;
}
// The challenge helpers take any transcript with verifier_bytes / a `sponge` member: the prover's
// Transcript and the verifier's VerifierTranscript (verifier.cu).
template <class F, class Ts>
inline F challenge(Ts& t) {
  return ChallengeCodec<F>::squeeze(t.sponge);
}
template <class F, class Ts>
inline std::vector<F> geometric_challenge(Ts& t, size_t count) {
  if (count == 0) return {};
  if (count == 1) return {F::one()};
  F x = challenge<F>(t);
  std::vector<F> r(count);
  r[0] = F::one();
  for (size_t i = 1; i < count; ++i) r[i] = r[i - 1] * x;
  return r;
}
// challenge_indices (src/protocols/challenge_indices.rs:6-50).
template <class Ts>
inline std::vector<uint64_t> challenge_indices(Ts& t, uint64_t num_leaves, size_t count, bool dedup) {
  if (count == 0) return {};
  if (num_leaves == 0 || (num_leaves & (num_leaves - 1))) throw Error(-1, "num_leaves must be a power of two");
  if (num_leaves == 1) return dedup ? std::vector<uint64_t>{0} : std::vector<uint64_t>(count, 0);
  int log = 0;
  while ((1ull << log) < num_leaves) ++log;
  size_t sb = (size_t)(log + 7) / 8;
  std::vector<uint8_t> ent(count * sb);
  t.verifier_bytes(ent.data(), ent.size());
  std::vector<uint64_t> idx(count);
  for (size_t i = 0; i < count; ++i) {
    uint64_t acc = 0;
    for (size_t k = 0; k < sb; ++k) acc = (acc << 8) | ent[i * sb + k];
    idx[i] = acc % num_leaves;
  }
  if (dedup) {
    std::sort(idx.begin(), idx.end());
    idx.erase(std::unique(idx.begin(), idx.end()), idx.end());
  }
  return idx;
}

// ---------------------------------------------------------------------------------------------
// Roots of unity (cooley_tukey.rs:51-127, NttEngine::new_from_fftfield): root(n) = g^((p-1)/n) for
// n dividing the engine order; extension engines use the same (lifted) roots.
//   Goldilocks g = 7, engine order 2^32 * 3   (fields.rs:85-91)
//   Field192   g = 3, engine order 2^48       (two-adicity 48, no small subgroup)
//   Field256   g = 5, engine order 2^28 * 3^2 (fields.rs:65-71)
// ---------------------------------------------------------------------------------------------
template <class B>
struct RootInfo;
template <>
struct RootInfo<Gl> {
  static uint64_t engine_order() { return 3ull << 32; }
  static Gl root(uint64_t n) { return Gl{gl_pow(7, (GL_P - 1) / n)}; }
  static constexpr int TABLE_LOG = 32;  // device root tables hold powers of root(2^32)
};
template <class P>
struct RootInfo<MontField<P>> {
  typedef MontField<P> M;
  static uint64_t engine_order() {
    return P::TWO_ADICITY >= 63 ? 0 : (P::SMALL_ORDER << P::TWO_ADICITY);
  }
  static M root(uint64_t n) {
    // (p - 1) / n by long division over the limbs, then g^quotient.
    uint64_t q[M::N];
    u128_t rem = 0;
    for (int i = M::N - 1; i >= 0; --i) {
      const uint64_t limb = i == 0 ? P::p(0) - 1 : P::p(i);
      const u128_t cur = (rem << 64) | limb;
      q[i] = (uint64_t)(cur / n);
      rem = cur % n;
    }
    uint64_t g[M::N] = {0};
    g[0] = P::GENERATOR;
    return M::from_canonical(g).pow_limbs(q, M::N);
  }
  static constexpr int TABLE_LOG = P::TWO_ADICITY < 32 ? P::TWO_ADICITY : 32;
};

template <class B>
inline B field_root(uint64_t n) {
  if (n == 0) return B::one();
  const uint64_t order = RootInfo<B>::engine_order();
  if (order % n != 0) throw Error(-1, "Subgroup of requested order does not exist.");
  return RootInfo<B>::root(n);
}
inline Gl gl_root(uint64_t n) { return field_root<Gl>(n); }

// evaluation_points with the default (transpose-permuted) order (cooley_tukey.rs:375-402).
template <class B>
inline std::vector<B> evaluation_points(uint64_t masked_len, uint64_t codeword_len, const std::vector<uint64_t>& idx) {
  if (masked_len > codeword_len) throw Error(-1, "masked length exceeds codeword length");
  if (codeword_len == 0 || (codeword_len & (codeword_len - 1))) throw Error(-2, "codeword length must be a power of two");
  uint64_t C = 1;
  while (C < masked_len) C <<= 1;
  uint64_t K = codeword_len / C;
  B g = field_root<B>(codeword_len);
  std::vector<B> res;
  for (uint64_t i : idx) {
    if (i >= codeword_len) throw Error(-1, "index out of range");
    uint64_t e = i / C + (i % C) * K;
    res.push_back(g.pow(e));
  }
  return res;
}

// ---------------------------------------------------------------------------------------------
// Configuration
// ---------------------------------------------------------------------------------------------
static constexpr double LOG2_10 = 3.32192809488736234787031942948939018;

struct Params {
  bool unique_decoding;
  size_t starting_log_inv_rate, initial_folding_factor, folding_factor, security_level, pow_bits, batch_size;
  uint8_t hash_id[32];
};

struct Pow {
  uint8_t hash_id[32];
  uint64_t threshold;
};

inline uint64_t pow_threshold(double bits) {
  if (!(bits >= 0.0 && bits <= 60.0)) throw Error(-1, "proof-of-work difficulty outside [0, 60] bits");
  double t = std::ceil(std::exp2(64.0 - bits));
  if (t >= 18446744073709551615.0) return UINT64_MAX;
  return (uint64_t)t;
}

struct Irs {
  size_t num_vectors, vector_size, mask_length, codeword_length, interleaving_depth, num_cols, layers;
  uint8_t hash_id[32];
  double johnson_slack;
  size_t in_domain_samples, out_domain_samples;
  bool dedup;
  double field_bits;
  size_t message_length() const { return vector_size / interleaving_depth; }
  size_t masked_message_length() const { return message_length() + mask_length; }
  double rate() const { return (double)masked_message_length() / (double)codeword_length; }
  bool unique_decoding() const { return out_domain_samples == 0 && johnson_slack == 0.0; }
  double list_size() const { return unique_decoding() ? 1.0 : 1. / (2. * johnson_slack * std::sqrt(rate())); }
  double rbr_queries() const {
    double per = unique_decoding() ? (1. + rate()) / 2. : std::sqrt(rate()) + johnson_slack;
    return (double)in_domain_samples * -std::log2(per);
  }
  double rbr_fold() const {
    double lir = -std::log2(rate());
    double lk = std::log2((double)masked_message_length());
    double err = unique_decoding() ? lk + lir : 7. * LOG2_10 + 3.5 * lir + 2. * lk;
    return field_bits - err;
  }
};

inline size_t layers_for(size_t n) {
  size_t l = 0;
  while (((size_t)1 << l) < n) ++l;
  return l;
}

inline Irs irs_new(double sec, bool ud, const uint8_t* hash_id, size_t nvec, size_t vsize, size_t depth, double rate,
                   double field_bits) {
  if (depth == 0 || vsize % depth) throw Error(-1, "vector size not divisible by interleaving depth");
  Irs c;
  size_t ml = vsize / depth;
  size_t cw = (size_t)std::ceil((double)ml / rate);
  double r = (double)ml / (double)cw;
  double js = ud ? 0.0 : std::sqrt(r) / 20.;
  size_t ood = 0;
  if (!ud) {
    double L = 1. / (2. * js * std::sqrt(r));
    double lc2 = L * (L - 1.) / 2.;
    double lps = field_bits - std::log2((double)(vsize - 1));
    if (!(lps > 0.)) throw Error(-1, "field too small for out-of-domain samples");
    ood = (size_t)std::max(std::ceil((sec + std::log2(lc2)) / lps), 1.);
  }
  double per = ud ? (1. + r) / 2. : std::sqrt(r) + js;
  c.num_vectors = nvec;
  c.vector_size = vsize;
  c.mask_length = 0;
  c.codeword_length = cw;
  c.interleaving_depth = depth;
  c.num_cols = depth * nvec;
  c.layers = layers_for(cw);
  memcpy(c.hash_id, hash_id, 32);
  c.johnson_slack = js;
  c.in_domain_samples = (size_t)std::ceil(sec / (-std::log2(per)));
  c.out_domain_samples = ood;
  c.dedup = false;
  c.field_bits = field_bits;
  return c;
}

struct Sumcheck {
  size_t initial_size, num_rounds, mask_length;
  Pow round_pow;
  size_t final_size() const {
    if (initial_size == 0 || num_rounds == 0) return initial_size;
    size_t p = 1;
    while (p < initial_size) p <<= 1;
    return p >> num_rounds;
  }
};

struct Round {
  Irs irs;
  Sumcheck sumcheck;
  Pow pow;
};

struct Config {
  int field;  // embedding id
  Irs initial;
  Sumcheck initial_sumcheck;
  Pow initial_skip_pow;
  std::vector<Round> rounds;
  Sumcheck final_sumcheck;
  Pow final_pow;
  size_t size() const { return initial.vector_size; }
};

// log2 of the field size: modulus limbs accumulated as f64 (most significant first), times the
// extension degree (fields.rs:10-30 field_size_bits).
inline double field_bits_of(int field) {
  double m = 0.0;
  int deg = 1;
  if (field >= 0 && field <= 2) {
    m = (double)GL_P;
    deg = field + 1;
  } else if (field == 4) {
    for (int i = F192Params::N - 1; i >= 0; --i) m = m * 18446744073709551616.0 + (double)F192Params::p(i);
  } else if (field == 5) {
    for (int i = F256Params::N - 1; i >= 0; --i) m = m * 18446744073709551616.0 + (double)F256Params::p(i);
  } else {
    throw Error(-1, "unknown field id");
  }
  return std::log2(m) * (double)deg;
}

inline Pow make_pow(const uint8_t* id, double bits) {
  Pow p;
  memcpy(p.hash_id, id, 32);
  p.threshold = pow_threshold(bits);
  return p;
}

inline Config config_new(int field, size_t size, const Params& wp) {
  if (size == 0 || (size & (size - 1))) throw Error(-1, "Only powers of two size are supported at the moment.");
  if (field < 0 || field > 5 || field == 3) throw Error(-1, "unknown field id");
  if (engine_kind(wp.hash_id) < 0) throw Error(-1, "unknown hash engine id");
  if (wp.batch_size == 0) throw Error(-1, "batch_size must be positive");
  Config cfg;
  cfg.field = field;
  const double fb = field_bits_of(field);
  const double sec = (double)wp.security_level;
  const double psec = (double)(wp.security_level > wp.pow_bits ? wp.security_level - wp.pow_bits : 0);
  size_t lir = wp.starting_log_inv_rate;
  size_t nv = layers_for(size);
  if (wp.initial_folding_factor > nv) throw Error(-1, "initial folding factor exceeds number of variables");
  cfg.initial = irs_new(psec, wp.unique_decoding, wp.hash_id, wp.batch_size, size, (size_t)1 << wp.initial_folding_factor,
                        std::pow(0.5, (int)wp.starting_log_inv_rate), fb);
  const Irs& ic = cfg.initial;
  double start_fold_bits = std::max(sec - std::min(ic.rbr_fold(), fb - std::log2(ic.list_size()) - 1.), 0.);
  double skip_bits = std::max(sec - (ic.rbr_fold() + std::log2((double)wp.initial_folding_factor)), 0.0);
  size_t round = 0, ids = ic.in_domain_samples;
  double qerr = ic.rbr_queries();
  nv -= wp.initial_folding_factor;
  while (nv >= wp.folding_factor) {
    size_t rff = round == 0 ? wp.initial_folding_factor : wp.folding_factor;
    size_t next_rate = lir + (rff - 1);
    Round rc;
    rc.irs = irs_new(psec, wp.unique_decoding, wp.hash_id, 1, (size_t)1 << nv, (size_t)1 << wp.folding_factor,
                     std::pow(0.5, (int)next_rate), fb);
    double ll = std::log2(rc.irs.list_size());
    double comb = fb - (std::log2((double)(rc.irs.out_domain_samples + ids)) + ll + 1.);
    double pow_bits = std::max(0., sec - std::min(qerr, comb));
    double fold_bits = std::max(sec - std::min(rc.irs.rbr_fold(), fb - (ll + 1.)), 0.);
    rc.sumcheck.initial_size = (size_t)1 << nv;
    rc.sumcheck.num_rounds = wp.folding_factor;
    rc.sumcheck.mask_length = 0;
    rc.sumcheck.round_pow = make_pow(wp.hash_id, fold_bits);
    rc.pow = make_pow(wp.hash_id, pow_bits);
    ++round;
    nv -= wp.folding_factor;
    lir = next_rate;
    ids = rc.irs.in_domain_samples;
    qerr = rc.irs.rbr_queries();
    cfg.rounds.push_back(rc);
  }
  double rbr = cfg.rounds.empty() ? ic.rbr_queries() : cfg.rounds.back().irs.rbr_queries();
  cfg.initial_sumcheck.initial_size = size;
  cfg.initial_sumcheck.num_rounds = wp.initial_folding_factor;
  cfg.initial_sumcheck.mask_length = 0;
  cfg.initial_sumcheck.round_pow = make_pow(wp.hash_id, start_fold_bits);
  cfg.initial_skip_pow = make_pow(wp.hash_id, skip_bits);
  cfg.final_sumcheck.initial_size = (size_t)1 << nv;
  cfg.final_sumcheck.num_rounds = nv;
  cfg.final_sumcheck.mask_length = 0;
  cfg.final_sumcheck.round_pow = make_pow(wp.hash_id, std::max(0., sec - fb + 1.0));
  cfg.final_pow = make_pow(wp.hash_id, std::max(0., sec - rbr));
  return cfg;
}

// CBOR of the configuration (ciborium::into_writer of whir::Config), hashed into the protocol id
// (SHA3-512).
inline std::vector<uint8_t> config_bytes(const Config& c);

}  // namespace whir

// Opaque handle of the C ABI: a derived WHIR configuration.
struct whir_config {
  whir::Config cfg;
};

namespace whir {

// CBOR (RFC 8949) writer with the encoding choices ciborium 0.2 makes for serde data: integers,
// lengths and tags in their shortest head; definite-length arrays, maps, byte and text strings;
// floats in the shortest of binary16 / binary32 / binary64 that keeps the value's exact bits.
struct CborWriter {
  std::vector<uint8_t> out;
  void head(unsigned major, uint64_t v) {
    const uint8_t m = (uint8_t)(major << 5);
    if (v < 24) {
      out.push_back(m | (uint8_t)v);
    } else if (v <= 0xff) {
      out.push_back(m | 24);
      out.push_back((uint8_t)v);
    } else if (v <= 0xffff) {
      out.push_back(m | 25);
      be(v, 2);
    } else if (v <= 0xffffffffull) {
      out.push_back(m | 26);
      be(v, 4);
    } else {
      out.push_back(m | 27);
      be(v, 8);
    }
  }
  void be(uint64_t v, int bytes) {
    for (int i = bytes - 1; i >= 0; --i) out.push_back((uint8_t)(v >> (8 * i)));
  }
  void uint(uint64_t v) { head(0, v); }
  void bytes(const uint8_t* b, size_t n) {
    head(2, n);
    out.insert(out.end(), b, b + n);
  }
  void text(const char* s) {
    const size_t n = strlen(s);
    head(3, n);
    out.insert(out.end(), s, s + n);
  }
  void array(size_t n) { head(4, n); }
  void map(size_t n) { head(5, n); }
  void boolean(bool b) { out.push_back(b ? 0xf5 : 0xf4); }
  // binary16 bits of d when d converts to binary16 exactly (finite values only).
  static bool to_half(double d, uint16_t* h) {
    if (!std::isfinite(d)) return false;
    const uint16_t sign = std::signbit(d) ? 0x8000 : 0;
    const double a = std::fabs(d);
    if (a == 0.0) {
      *h = sign;
      return true;
    }
    int e;
    const double m = std::frexp(a, &e);  // a = m * 2^e, m in [0.5, 1)
    // normal binary16: a = (1 + f / 1024) * 2^(E - 15), E in [1, 30]  <=>  e - 1 = E - 15
    const int E = e - 1 + 15;
    if (E >= 1 && E <= 30) {
      const double f = (m * 2.0 - 1.0) * 1024.0;
      if (f != std::floor(f)) return false;
      *h = (uint16_t)(sign | (E << 10) | (uint16_t)f);
      return true;
    }
    if (E < 1) {  // subnormal: a = f * 2^-24, f in [1, 1023]
      const double f = std::ldexp(a, 24);
      if (f != std::floor(f) || f < 1.0 || f > 1023.0) return false;
      *h = (uint16_t)(sign | (uint16_t)f);
      return true;
    }
    return false;
  }
  void f64(double d) {
    uint16_t h;
    if (to_half(d, &h)) {
      out.push_back(0xf9);
      be(h, 2);
      return;
    }
    const float f = (float)d;
    if (std::isfinite(d) && (double)f == d) {
      uint32_t b;
      memcpy(&b, &f, 4);
      out.push_back(0xfa);
      be(b, 4);
      return;
    }
    uint64_t b;
    memcpy(&b, &d, 8);
    out.push_back(0xfb);
    be(b, 8);
  }
};

// The serde data model of whir::Config<M> (protocols/whir/mod.rs:29-46) as ciborium::into_writer
// writes it for the protocol id (transcript/mod.rs:111-121): structs are maps keyed by their field
// names in declaration order; EngineId ([u8; 32] newtype) is an array of 32 integers; usize and u64
// are unsigned integers; OrderedFloat<f64> is a float; Typed<M> is {"type": M's type info, "value":
// M} (type_info.rs:98-117); a field's type info is FieldInfo {characteristic: big-endian bytes
// without leading zeros, extension_degree} (fields.rs:32-62); embeddings serialize their one Type
// field ("field" for Identity, "extension" for Basefield, embedding.rs:43-59, 191-205).
inline void cbor_field_info(CborWriter& w, int base_field, size_t degree) {
  std::vector<uint8_t> le;
  if (base_field == 4 || base_field == 5) {
    const int n = base_field == 4 ? F192Params::N : F256Params::N;
    for (int i = 0; i < n; ++i) {
      const uint64_t limb = base_field == 4 ? F192Params::p(i) : F256Params::p(i);
      for (int b = 0; b < 8; ++b) le.push_back((uint8_t)(limb >> (8 * b)));
    }
  } else {
    for (int b = 0; b < 8; ++b) le.push_back((uint8_t)(GL_P >> (8 * b)));
  }
  while (!le.empty() && le.back() == 0) le.pop_back();
  std::vector<uint8_t> bev(le.rbegin(), le.rend());
  w.map(2);
  w.text("characteristic");
  w.bytes(bev.data(), bev.size());
  w.text("extension_degree");
  w.uint(degree);
}
// Base prime field and extension degree of an embedding id's target field.
inline void field_parts(int field, int* base, size_t* degree) {
  if (field >= 0 && field <= 2) {
    *base = 0;
    *degree = (size_t)field + 1;
  } else {
    *base = field;
    *degree = 1;
  }
}
inline void cbor_engine(CborWriter& w, const uint8_t* id) {
  w.array(32);
  for (int i = 0; i < 32; ++i) w.uint(id[i]);
}
inline void cbor_pow(CborWriter& w, const Pow& p) {
  w.map(2);
  w.text("hash_id");
  cbor_engine(w, p.hash_id);
  w.text("threshold");
  w.uint(p.threshold);
}
inline void cbor_sumcheck(CborWriter& w, const Sumcheck& s, int field) {
  int base;
  size_t degree;
  field_parts(field, &base, &degree);
  w.map(5);
  w.text("field");
  cbor_field_info(w, base, degree);
  w.text("initial_size");
  w.uint(s.initial_size);
  w.text("round_pow");
  cbor_pow(w, s.round_pow);
  w.text("num_rounds");
  w.uint(s.num_rounds);
  w.text("mask_length");
  w.uint(s.mask_length);
}
// irs_commit::Config<M> (irs_commit.rs:51-91) for the embedding `field` (basefield: the initial
// committer of an extension-field config), or the identity embedding of the target field (rounds).
inline void cbor_irs(CborWriter& w, const Irs& r, int field, bool identity) {
  int base;
  size_t degree;
  field_parts(field, &base, &degree);
  const bool basefield = !identity && degree > 1;
  w.map(11);
  w.text("embedding");
  w.map(2);
  w.text("type");
  w.text(basefield ? "basefield" : "identity");
  w.text("value");
  w.map(1);
  w.text(basefield ? "extension" : "field");
  cbor_field_info(w, base, degree);
  w.text("num_vectors");
  w.uint(r.num_vectors);
  w.text("vector_size");
  w.uint(r.vector_size);
  w.text("mask_length");
  w.uint(r.mask_length);
  w.text("codeword_length");
  w.uint(r.codeword_length);
  w.text("interleaving_depth");
  w.uint(r.interleaving_depth);
  w.text("matrix_commit");  // matrix_commit::Config (matrix_commit.rs:93-111), with_hash
  w.map(4);
  w.text("element_type");
  cbor_field_info(w, base, basefield ? 1 : degree);
  w.text("num_cols");
  w.uint(r.num_cols);
  w.text("leaf_hash_id");
  cbor_engine(w, r.hash_id);
  w.text("merkle_tree");  // merkle_tree::Config (merkle_tree.rs:25-40)
  w.map(2);
  w.text("num_leaves");
  w.uint(r.codeword_length);
  w.text("layers");
  w.array(r.layers);
  for (size_t l = 0; l < r.layers; ++l) {
    w.map(1);
    w.text("hash_id");
    cbor_engine(w, r.hash_id);
  }
  w.text("johnson_slack");
  w.f64(r.johnson_slack);
  w.text("in_domain_samples");
  w.uint(r.in_domain_samples);
  w.text("out_domain_samples");
  w.uint(r.out_domain_samples);
  w.text("deduplicate_in_domain");
  w.boolean(r.dedup);
}

// CBOR of the configuration: the bytes whose SHA3-512 is the protocol id.
inline std::vector<uint8_t> config_bytes(const Config& c) {
  CborWriter w;
  w.map(6);
  w.text("initial_committer");
  cbor_irs(w, c.initial, c.field, false);
  w.text("initial_sumcheck");
  cbor_sumcheck(w, c.initial_sumcheck, c.field);
  w.text("initial_skip_pow");
  cbor_pow(w, c.initial_skip_pow);
  w.text("round_configs");
  w.array(c.rounds.size());
  for (const Round& r : c.rounds) {
    w.map(3);
    w.text("irs_committer");
    cbor_irs(w, r.irs, c.field, true);
    w.text("sumcheck");
    cbor_sumcheck(w, r.sumcheck, c.field);
    w.text("pow");
    cbor_pow(w, r.pow);
  }
  w.text("final_sumcheck");
  cbor_sumcheck(w, c.final_sumcheck, c.field);
  w.text("final_pow");
  cbor_pow(w, c.final_pow);
  return w.out;
}

}  // namespace whir
