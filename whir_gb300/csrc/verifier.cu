// Host-side WHIR verifier of the C ABI: whir_verify (include/whir_gb300.h).
//
// Restates whir::Config::verify (reference src/protocols/whir/verifier.rs:45-265) with the
// library's own transcript, codecs and configuration, followed by FinalClaim::verify
// (src/protocols/whir/mod.rs:63-74) against the statement's linear forms. The pieces it checks:
//   commitments  irs_commit::Config::receive_commitment (irs_commit.rs:438-451): root, OOD points/values
//   openings     irs_commit::Config::verify (irs_commit.rs:453-484): query indices, opened rows (hints),
//                leaf digests and Merkle authentication paths (merkle_tree.rs:188-273)
//   sumchecks    protocols/sumcheck.rs:165-215 (round messages, round PoW, folding challenges)
//   PoW          proof_of_work.rs:168-191
// Verification is O(queries x log N) hashing and field work on the host; it needs no GPU.
#include <algorithm>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/whir_gb300.h"
#include "field.cuh"
#include "hash.cuh"
#include "protocol.hpp"
#include "sponge.cuh"

using namespace whir;

namespace {

thread_local std::string g_verify_error;

struct Reject {
  const char* why;
};

// Verifier side of the transcript: prover messages are read from the NARG string and absorbed,
// challenges are squeezed, hints are read from the hint string without touching the sponge.
struct VerifierTranscript {
  Sponge sponge;
  const uint8_t* narg;
  size_t narg_len, narg_pos = 0;
  const uint8_t* hints;
  size_t hints_len, hints_pos = 0;
  void prover_bytes(uint8_t* out, size_t n) {
    if (narg_len - narg_pos < n) throw Reject{"proof string too short"};
    memcpy(out, narg + narg_pos, n);
    narg_pos += n;
    sponge.absorb(out, n);
  }
  void verifier_bytes(uint8_t* out, size_t n) { sponge.squeeze(out, n); }
  void hint_bytes(uint8_t* out, size_t n) {
    if (hints_len - hints_pos < n) throw Reject{"hint string too short"};
    memcpy(out, hints + hints_pos, n);
    hints_pos += n;
  }
};

template <class F>
F parse_elem(const uint8_t* b) {
  uint64_t c[F::LIMBS];
  for (int d = 0; d < F::LIMBS; ++d) {
    c[d] = 0;
    for (int i = 7; i >= 0; --i) c[d] = (c[d] << 8) | b[8 * d + i];
  }
  if (!Canon<F>::ok(c)) throw Reject{"non-canonical field element"};
  return Canon<F>::from(c);
}
template <class F>
F recv_elem(VerifierTranscript& vt) {
  uint8_t b[8 * F::LIMBS];
  vt.prover_bytes(b, sizeof(b));
  return parse_elem<F>(b);
}

void pow_check(const Pow& p, VerifierTranscript& vt) {
  if (p.threshold == UINT64_MAX) return;
  const int kind = engine_kind(p.hash_id);
  if (kind < 0 || kind == HASH_COPY) throw Reject{"proof-of-work engine cannot hash 64-byte inputs"};
  uint8_t chal[32], nonce[8], in[64] = {0}, out[32];
  vt.verifier_bytes(chal, 32);
  vt.prover_bytes(nonce, 8);
  memcpy(in, chal, 32);
  memcpy(in + 32, nonce, 8);
  host_hash(kind, in, 64, out);
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | out[i];
  if (v > p.threshold) throw Reject{"proof of work above threshold"};
}

template <class F>
std::vector<F> sumcheck_check(const Sumcheck& c, VerifierTranscript& vt, F& sum) {
  std::vector<F> rs;
  for (size_t round = 0; round < c.num_rounds; ++round) {
    const F u0 = recv_elem<F>(vt), u2 = recv_elem<F>(vt);
    const F u1 = sum - u0.dbl() - u2;
    pow_check(c.round_pow, vt);
    const F r = challenge<F>(vt);
    rs.push_back(r);
    sum = (u2 * r + u1) * r + u0;
  }
  return rs;
}

struct Digest {
  uint8_t b[32];
  bool operator==(const Digest& o) const { return !memcmp(b, o.b, 32); }
};

// Recomputes the root from the queried leaves and the sibling hints (sorted distinct indices, one
// layer at a time; a sibling is read only when it is not itself a queried node).
Digest merkle_root(int kind, size_t layers, std::vector<std::pair<uint64_t, Digest>> leaves, VerifierTranscript& vt) {
  std::stable_sort(leaves.begin(), leaves.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  std::vector<uint64_t> idx;
  std::vector<Digest> hs;
  for (size_t i = 0; i < leaves.size(); ++i) {
    if (i > 0 && leaves[i].first == leaves[i - 1].first) {
      if (!(leaves[i].second == leaves[i - 1].second)) throw Reject{"one leaf opened to two different rows"};
      continue;
    }
    idx.push_back(leaves[i].first);
    hs.push_back(leaves[i].second);
  }
  for (size_t l = 0; l < layers; ++l) {
    std::vector<uint64_t> next_idx;
    std::vector<Digest> next_hs;
    for (size_t i = 0; i < idx.size(); ++i) {
      const uint64_t a = idx[i];
      uint8_t msg[64];
      if (i + 1 < idx.size() && idx[i + 1] == (a ^ 1)) {
        memcpy(msg, hs[i].b, 32);
        memcpy(msg + 32, hs[i + 1].b, 32);
        ++i;
      } else {
        Digest sib;
        vt.hint_bytes(sib.b, 32);
        memcpy(msg, (a & 1) ? sib.b : hs[i].b, 32);
        memcpy(msg + 32, (a & 1) ? hs[i].b : sib.b, 32);
      }
      Digest parent;
      host_hash(kind, msg, 64, parent.b);
      next_idx.push_back(a >> 1);
      next_hs.push_back(parent);
    }
    idx.swap(next_idx);
    hs.swap(next_hs);
  }
  if (hs.size() != 1) throw Reject{"malformed authentication paths"};
  return hs[0];
}

template <class T>
struct Commitment {
  Digest root;
  std::vector<T> ood_points, ood_values;  // ood_values: samples x vectors
};

template <class T>
Commitment<T> receive_commitment(const Irs& c, VerifierTranscript& vt) {
  Commitment<T> cm;
  vt.prover_bytes(cm.root.b, 32);
  for (size_t i = 0; i < c.out_domain_samples; ++i) cm.ood_points.push_back(challenge<T>(vt));
  for (size_t i = 0; i < c.out_domain_samples * c.num_vectors; ++i) cm.ood_values.push_back(recv_elem<T>(vt));
  return cm;
}

// Opened rows (points x (commitments * num_cols)), checked against each commitment's root.
template <class S, class T>
void open_check(const Irs& c, VerifierTranscript& vt, const std::vector<const Commitment<T>*>& cms,
                std::vector<T>& points, std::vector<T>& rows) {
  const int kind = engine_kind(c.hash_id);
  if (kind < 0) throw Reject{"unknown leaf hash engine"};
  std::vector<uint64_t> idx = challenge_indices(vt, c.codeword_length, c.in_domain_samples, c.dedup);
  points.clear();
  for (const auto& p : evaluation_points<typename S::Base>(c.masked_message_length(), c.codeword_length, idx))
    points.push_back(T::from_base(p));
  const size_t q = idx.size(), nc = c.num_cols, stride = cms.size() * nc;
  rows.assign(q * stride, T::zero());
  for (size_t k = 0; k < cms.size(); ++k) {
    uint8_t lb[8];
    vt.hint_bytes(lb, 8);
    uint64_t n = 0;
    for (int i = 7; i >= 0; --i) n = (n << 8) | lb[i];
    if (n != q * nc) throw Reject{"opened submatrix has the wrong size"};
    std::vector<uint8_t> row(nc * 8 * S::LIMBS);
    std::vector<std::pair<uint64_t, Digest>> leaves;
    for (size_t pi = 0; pi < q; ++pi) {
      vt.hint_bytes(row.data(), row.size());
      for (size_t j = 0; j < nc; ++j)
        rows[pi * stride + k * nc + j] = Embed<T, S>::map(parse_elem<S>(row.data() + j * 8 * S::LIMBS));
      Digest leaf;
      host_hash(kind, row.data(), row.size(), leaf.b);
      leaves.push_back({idx[pi], leaf});
    }
    if (!(merkle_root(kind, c.layers, leaves, vt) == cms[k]->root)) throw Reject{"Merkle root mismatch"};
  }
}

template <class T>
std::vector<T> eq_weights(const std::vector<T>& point) {
  std::vector<T> t{T::one()};
  for (const T& x : point) {
    std::vector<T> nt(t.size() * 2);
    for (size_t b = 0; b < t.size(); ++b) {
      const T s1 = t[b] * x;
      nt[2 * b] = t[b] - s1;
      nt[2 * b + 1] = s1;
    }
    t.swap(nt);
  }
  return t;
}

// eq(point, .) paired with the point's variables consumed from the last (univariate_evaluation.rs:44-53):
// the multilinear extension of (x^i)_i at `point`.
template <class T>
T univariate_mle(const T& x, const std::vector<T>& point) {
  T x2i = x, res = T::one();
  for (size_t k = point.size(); k-- > 0;) {
    const T& r = point[k];
    res = res * ((T::one() - r) + r * x2i);
    x2i = x2i * x2i;
  }
  return res;
}

template <class T>
T mle_of_eq(const std::vector<T>& l, const std::vector<T>& r) {
  T acc = T::one();
  for (size_t i = 0; i < l.size(); ++i) acc = acc * (l[i] * r[i] + (T::one() - l[i]) * (T::one() - r[i]));
  return acc;
}

template <class S, class T>
void verify_impl(const Config& cfg, VerifierTranscript& vt, size_t n_commitments,
                 const std::vector<std::vector<T>>& mle_points, const std::vector<std::vector<T>>& covectors,
                 const std::vector<T>& evaluations) {
  const size_t nv = n_commitments * cfg.initial.num_vectors;
  const size_t nforms = mle_points.size() + covectors.size();
  if (evaluations.size() != nv * nforms) throw Reject{"evaluation matrix size mismatch"};
  std::vector<Commitment<T>> cms;
  for (size_t k = 0; k < n_commitments; ++k) cms.push_back(receive_commitment<T>(cfg.initial, vt));
  if (nv == 0) return;

  // Out-of-domain cross terms (prover.rs:98-128).
  std::vector<T> oods_points, oods_matrix;
  size_t voff = 0;
  for (const auto& cm : cms) {
    const size_t wn = cfg.initial.num_vectors;
    for (size_t oi = 0; oi < cm.ood_points.size(); ++oi) {
      for (size_t j = 0; j < nv; ++j)
        oods_matrix.push_back(j >= voff && j < voff + wn ? cm.ood_values[oi * wn + (j - voff)] : recv_elem<T>(vt));
      oods_points.push_back(cm.ood_points[oi]);
    }
    voff += wn;
  }
  const std::vector<T> vector_rlc = geometric_challenge<T>(vt, nv);
  const std::vector<T> constraint_rlc = geometric_challenge<T>(vt, nforms + oods_points.size());
  const std::vector<T> init_rlc(constraint_rlc.begin(), constraint_rlc.begin() + nforms);
  const std::vector<T> oods_rlc(constraint_rlc.begin() + nforms, constraint_rlc.end());
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
  struct Constraints {
    std::vector<T> rlc, points;
    size_t size;
  };
  std::vector<Constraints> constraints{{oods_rlc, oods_points, cfg.size()}};
  std::vector<std::vector<T>> round_folding;
  std::vector<T> folding;
  if (constraint_rlc.empty()) {
    if (!the_sum.is_zero()) throw Reject{"nonzero claim without constraints"};
    for (size_t i = 0; i < cfg.initial_sumcheck.num_rounds; ++i) folding.push_back(challenge<T>(vt));
    pow_check(cfg.initial_skip_pow, vt);
  } else {
    folding = sumcheck_check<T>(cfg.initial_sumcheck, vt, the_sum);
  }
  round_folding.push_back(folding);

  std::vector<const Commitment<T>*> initial_cms;
  for (const auto& cm : cms) initial_cms.push_back(&cm);
  Commitment<T> prev;
  bool have_prev = false;
  std::vector<T> poly_rlc;
  // Opens the previous commitment (the initial ones first) and returns its points and rows.
  auto open_prev = [&](size_t ri, std::vector<T>& pts, std::vector<T>& rows) {
    if (!have_prev) {
      open_check<S, T>(cfg.initial, vt, initial_cms, pts, rows);
      poly_rlc = vector_rlc;
    } else {
      open_check<T, T>(cfg.rounds[ri - 1].irs, vt, std::vector<const Commitment<T>*>{&prev}, pts, rows);
      poly_rlc = {T::one()};
    }
  };
  auto row_values = [&](const std::vector<T>& pts, const std::vector<T>& rows) {
    const std::vector<T> eqw = eq_weights(round_folding.back());
    std::vector<T> wts;
    for (const T& x : poly_rlc)
      for (const T& y : eqw) wts.push_back(x * y);
    std::vector<T> vals;
    const size_t cols = pts.empty() ? 0 : rows.size() / pts.size();
    if (cols != wts.size()) throw Reject{"opened row width mismatch"};
    for (size_t pi = 0; pi < pts.size(); ++pi) {
      T acc = T::zero();
      for (size_t k = 0; k < cols; ++k) acc += wts[k] * rows[pi * cols + k];
      vals.push_back(acc);
    }
    return vals;
  };
  for (size_t ri = 0; ri < cfg.rounds.size(); ++ri) {
    const Round& rc = cfg.rounds[ri];
    Commitment<T> cm = receive_commitment<T>(rc.irs, vt);
    pow_check(rc.pow, vt);
    std::vector<T> pts, rows;
    open_prev(ri, pts, rows);
    std::vector<T> all_points = cm.ood_points;
    all_points.insert(all_points.end(), pts.begin(), pts.end());
    std::vector<T> vals;
    for (size_t o = 0; o < cm.ood_points.size(); ++o) vals.push_back(cm.ood_values[o]);
    const std::vector<T> in_vals = row_values(pts, rows);
    vals.insert(vals.end(), in_vals.begin(), in_vals.end());
    const std::vector<T> rlc = geometric_challenge<T>(vt, vals.size());
    for (size_t k = 0; k < vals.size(); ++k) the_sum += rlc[k] * vals[k];
    constraints.push_back({rlc, all_points, rc.irs.vector_size});
    folding = sumcheck_check<T>(rc.sumcheck, vt, the_sum);
    round_folding.push_back(folding);
    prev = std::move(cm);
    have_prev = true;
  }
  std::vector<T> final_vector;
  for (size_t i = 0; i < cfg.final_sumcheck.initial_size; ++i) final_vector.push_back(recv_elem<T>(vt));
  pow_check(cfg.final_pow, vt);
  {
    std::vector<T> pts, rows;
    open_prev(cfg.rounds.size(), pts, rows);
    const std::vector<T> expect = row_values(pts, rows);
    for (size_t pi = 0; pi < pts.size(); ++pi) {
      T got = T::zero();
      for (size_t k = final_vector.size(); k-- > 0;) got = got * pts[pi] + final_vector[k];
      if (got != expect[pi]) throw Reject{"final vector disagrees with an opened row"};
    }
  }
  const std::vector<T> fin = sumcheck_check<T>(cfg.final_sumcheck, vt, the_sum);
  round_folding.push_back(fin);
  std::vector<T> evaluation_point;
  for (const auto& r : round_folding) evaluation_point.insert(evaluation_point.end(), r.begin(), r.end());
  // The final vector's multilinear extension at the last sumcheck's randomness.
  T poly_eval = T::zero();
  {
    const std::vector<T> eqw = eq_weights(fin);
    for (size_t i = 0; i < final_vector.size() && i < eqw.size(); ++i) poly_eval += eqw[i] * final_vector[i];
  }
  if (poly_eval.is_zero()) throw Reject{"final polynomial evaluates to zero"};
  T lf_rlc = the_sum * poly_eval.inv();
  for (const auto& cs : constraints) {
    const size_t num_vars = layers_for(cs.size);
    const size_t start = evaluation_point.size() >= num_vars ? evaluation_point.size() - num_vars : 0;
    const std::vector<T> tail(evaluation_point.begin() + start, evaluation_point.end());
    for (size_t k = 0; k < cs.points.size(); ++k) lf_rlc -= cs.rlc[k] * univariate_mle(cs.points[k], tail);
  }
  // FinalClaim::verify: the random combination of the statement's forms at the evaluation point.
  T acc = T::zero();
  size_t k = 0;
  for (const auto& pt : mle_points) acc += init_rlc[k++] * mle_of_eq(pt, evaluation_point);
  for (const auto& cv : covectors) {
    const std::vector<T> eqw = eq_weights(evaluation_point);
    T m = T::zero();
    for (size_t i = 0; i < cv.size() && i < eqw.size(); ++i) m += eqw[i] * cv[i];
    acc += init_rlc[k++] * m;
  }
  if (acc != lf_rlc) throw Reject{"final claim does not match the statement"};
}

template <class T>
std::vector<T> load_elems(const uint64_t* p, size_t n) {
  std::vector<T> v(n);
  for (size_t i = 0; i < n; ++i) {
    if (!Canon<T>::ok(p + i * T::LIMBS)) throw Error(WHIR_ERR_INVALID, "non-canonical field element");
    v[i] = Canon<T>::from(p + i * T::LIMBS);
  }
  return v;
}

}  // namespace

extern "C" {

const char* whir_verify_last_reason(void) { return g_verify_error.c_str(); }

int whir_verify(const whir_config* cfg, const char* session, size_t session_len, const uint8_t* narg,
                size_t narg_len, const uint8_t* hints, size_t hints_len, size_t n_commitments,
                const uint64_t* mle_points, size_t n_points, const uint64_t* covectors, size_t n_covectors,
                const uint64_t* evaluations) {
  g_verify_error.clear();
  try {
    if (!cfg || (narg_len && !narg) || (hints_len && !hints)) throw Error(WHIR_ERR_INVALID, "null argument");
    const Config& c = cfg->cfg;
    const size_t n = c.size(), nvars = layers_for(n), nv = n_commitments * c.initial.num_vectors;
    auto run = [&](auto s_tag, auto t_tag) {
      typedef decltype(s_tag) S;
      typedef decltype(t_tag) T;
      std::vector<std::vector<T>> pts, covs;
      for (size_t i = 0; i < n_points; ++i) pts.push_back(load_elems<T>(mle_points + i * nvars * T::LIMBS, nvars));
      for (size_t i = 0; i < n_covectors; ++i) covs.push_back(load_elems<T>(covectors + i * n * T::LIMBS, n));
      const size_t ne = (n_points + n_covectors) * nv;
      std::vector<T> evals = ne ? load_elems<T>(evaluations, ne) : std::vector<T>();
      VerifierTranscript vt;
      vt.sponge.reset();
      std::vector<uint8_t> cb = config_bytes(c);
      uint8_t pid[64], sid[32];
      sha3_512_host(cb.data(), cb.size(), pid);
      std::vector<uint8_t> st = cbor_text(std::string(session ? session : "", session ? session_len : 0));
      sha3_256_host(st.data(), st.size(), sid);
      vt.sponge.absorb(pid, 64);
      vt.sponge.absorb(sid, 32);
      vt.narg = narg;
      vt.narg_len = narg_len;
      vt.hints = hints;
      vt.hints_len = hints_len;
      verify_impl<S, T>(c, vt, n_commitments, pts, covs, evals);
      if (vt.narg_pos != narg_len || vt.hints_pos != hints_len) throw Reject{"trailing proof bytes"};
    };
    switch (c.field) {
      case WHIR_GOLDILOCKS1: run(Gl{}, Gl{}); break;
      case WHIR_GOLDILOCKS2: run(Gl{}, Gl2{}); break;
      case WHIR_GOLDILOCKS3: run(Gl{}, Gl3{}); break;
      case WHIR_FIELD192: run(F192{}, F192{}); break;
      case WHIR_FIELD256: run(F256{}, F256{}); break;
      default: throw Error(WHIR_ERR_INVALID, "unknown field id");
    }
    return 0;
  } catch (const Reject& r) {
    g_verify_error = r.why;
    return WHIR_REJECT;
  } catch (const Error& e) {
    g_verify_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_verify_error = e.what();
    return WHIR_ERR_INTERNAL;
  }
}

}  // extern "C"
