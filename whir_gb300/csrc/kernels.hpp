// Launchers for the sm_103a kernels of the WHIR prover path. Every launcher enqueues work on the
// given stream and returns a cudaError_t (or a negative WHIR status for unsupported shapes); none
// of them synchronizes.
#pragma once
#include <algorithm>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "field.cuh"

namespace whir {

// Process-wide count of kernel launches issued by this library (instrumentation only).
uint64_t kernel_launches();
void note_launch();

// Powers of the 2^log_order-th root of unity w of a base prime field, stored as base-field elements
// (Montgomery form for Field192/Field256): lo[i] = w^i (i < 2^16), hi[i] = w^(i * 2^16)
// (i < 2^(log_order - 16)). ntt: the in-CTA NTT twiddles by level, level L = 1..NTT_TW_LEVELS
// holding w_(2^L)^q for q < 2^(L-1) at offset 2^(L-1) - 1.
static constexpr int NTT_TW_LEVELS = 12;
struct RootTab {
  const uint64_t* lo;
  const uint64_t* hi;
  const uint64_t* ntt;
  int log_order;
};

// Where a kernel publishes a small result for a host that polls host-mapped memory: `data` receives
// the bytes, flag[1] the context's device error word (*dev_err), then flag[0] = seq after a
// system-wide fence.
struct MailSlot {
  uint8_t* data = nullptr;
  unsigned int* flag = nullptr;
  unsigned int seq = 0;
  const unsigned int* dev_err = nullptr;
};

// In-place conversion between the canonical limbs of the C ABI and the in-memory form of F
// (a no-op for the Goldilocks family; Montgomery form for Field192/Field256).
template <class F>
cudaError_t launch_to_internal(F* v, size_t n, cudaStream_t s);
template <class F>
cudaError_t launch_to_canonical(F* v, size_t n, cudaStream_t s);

// Shape of one interleaved Reed–Solomon encode (reference cooley_tukey.rs:411-477).
struct EncodePlan {
  int mode;          // 0: single pass (cosets_per_cta cosets per CTA); 1: four-step (two passes)
  int logC, logN;    // coset size and codeword length (powers of two)
  int logC1, logC2;  // four-step split C = C1 * C2
  int cosets_per_cta;
  int cols_per_cta;  // four-step pass 1 width
  size_t scratch_elems;  // intermediate elements needed by mode 1
};

// Plans an encode of n_msgs messages of msg_len elements (elem_bytes each) into codeword_len rows:
// the autotuned choice for the shape when one is recorded (encode_tuning_set), else the default
// heuristics (plan_encode_default). Returns 0, or a negative status when the shape is unsupported.
int plan_encode(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t elem_bytes, EncodePlan* plan);
int plan_encode_default(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t elem_bytes, EncodePlan* plan);
// Explicit plan choices: mode 0 with G cosets per CTA, or mode 1 with a 2^logC2-point row pass and
// W columns per column-pass CTA.
struct EncodeTuning {
  int mode, logC2, W, G;
};
// Largest NTT an encode CTA runs in shared memory (log2 points): a four-step pass transforms at most
// 2^ENC_MAX_NTT_LOG points.
static constexpr int ENC_MAX_NTT_LOG = 12;
int plan_encode_tuned(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t elem_bytes, const EncodeTuning& t,
                      EncodePlan* plan);
// Process-wide table of tuned choices (encode plans by shape, Merkle tile heights by tree height),
// written by the autotuner, exported and imported as text lines
//   "encode <n_msgs> <msg_len> <codeword_len> <elem_bytes> <mode> <logC2> <W> <G>"
//   "merkle <layers> <tile_log>"
void encode_tuning_set(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t elem_bytes, const EncodeTuning& t);
bool encode_tuning_get(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t elem_bytes, EncodeTuning* t);
void merkle_tuning_set(int layers, int tile_log);
int merkle_tile_log_for(int layers);
std::string tuning_export();
int tuning_import(const char* text);
void tuning_clear();

// Messages made resident by work on another stream, in `groups` consecutive message groups:
// group g holds messages [bounds[g], bounds[g + 1]) (bounds[0] = 0, bounds[groups] = n_msgs), and
// ready[g] is recorded once they are in place. The encode waits for each group's event just before
// the first kernel that reads it, so the column passes of earlier groups overlap the copies of
// later ones.
struct EncodeStaging {
  int groups;
  const size_t* bounds;
  const cudaEvent_t* ready;
};

// Encodes messages (n_msgs x msg_len, message-major) into dst (codeword_len x n_msgs, row-major).
// When leaves != nullptr, also writes the digest of every row (canonical LE bytes of its elements)
// with engine `hash_kind`. scratch must hold plan.scratch_elems elements.
template <class F>
cudaError_t launch_encode(const EncodePlan& plan, const F* src, size_t n_msgs, size_t msg_len, F* dst,
                          uint32_t* leaves, int hash_kind, F* scratch, RootTab rt, cudaStream_t s,
                          const EncodeStaging* staging = nullptr);

// Four-step pass 1 of one message of one coset (plan.mode == 1, codeword length = coset size) from
// its nonzero coefficients grouped by column: column q is j2 = col_j2[q] with entries
// [col_off[q], col_off[q + 1]) of (ent_j1, ent_val) (coefficient index j1 * C2 + j2). Writes those
// columns of the intermediate `inter` (plan.scratch_elems elements), whose other entries the caller
// zeroes; launch_encode_rows_pass then finishes the transform.
template <class F>
cudaError_t launch_sparse_cols(const EncodePlan& plan, const uint32_t* col_j2, const uint32_t* col_off,
                               const uint32_t* ent_j1, const F* ent_val, size_t ncols, F* inter, RootTab rt,
                               cudaStream_t s);
template <class F>
cudaError_t launch_encode_rows_pass(const EncodePlan& plan, const F* scratch, size_t n_msgs, size_t msg_len, F* dst,
                                    RootTab rt, cudaStream_t s, size_t add_rows = 0);

// Several independent interleaved encodes (jobs of possibly different shapes, one field) in one
// launch per pass: the CTAs of a launch are split among the jobs by a device table of per-job
// arguments (encode_multi_prepare fills its host image; upload it, then launch_encode_multi).
struct EncodeJobDesc {
  EncodePlan plan;
  const void* src;   // messages (device, message-major)
  size_t n_msgs, msg_len;
  void* dst;         // codeword (device, row-major)
  uint32_t* leaves;  // leaf digests (device), or nullptr
  void* scratch;     // four-step intermediate of plan.scratch_elems elements (mode 1 jobs)
};
struct EncodeMultiLaunch {
  int ncols, nrows;             // jobs in the column pass (four-step jobs) and in the row pass
  uint64_t cols_grid, rows_grid;
  size_t cols_smem, rows_smem;  // dynamic shared memory (the largest job's)
  size_t rows_off, bytes;       // byte offset of the row-pass table in the image; image size
};
template <class F>
size_t encode_multi_table_bytes(size_t njobs);
template <class F>
int encode_multi_prepare(const EncodeJobDesc* jobs, size_t njobs, RootTab rt, void* host_image,
                         EncodeMultiLaunch* out);
template <class F>
cudaError_t launch_encode_multi(const EncodeMultiLaunch& l, const void* dev_image, int hash_kind, cudaStream_t s);

// Merkle trees of several jobs built together: each launch covers the tiles of every tree at the
// same step (merkle_multi_plan lays out the table image to upload; launch_merkle_multi runs it).
struct MerkleJobDesc {
  uint32_t* nodes;
  int layers;
};
struct MerkleMultiLaunch {
  size_t offset;  // byte offset of the launch's table slice in the image
  int n, S;       // trees in the launch, phase-A depth
  uint64_t grid;
};
void merkle_multi_plan(const MerkleJobDesc* jobs, size_t njobs, int tile_log, std::vector<MerkleMultiLaunch>& launches,
                       std::vector<uint8_t>& image);
cudaError_t launch_merkle_multi(const std::vector<MerkleMultiLaunch>& launches, const void* dev_image, int hash_kind,
                                cudaStream_t s);

// Builds Merkle layers above the leaf layer in place. nodes: (2^(layers+1) - 1) digests laid out
// [leaves (2^layers)][layer 1]...[root] (merkle_tree.rs:96-121). Each launch hashes tiles of
// 2^tile_log nodes up tile_log layers (tile_log <= 0: the tuned height for this tree, or
// merkle_tile_log, 10, when none is recorded).
// When mail.data is set (layers >= 1), the launch that computes the root also publishes it (32 bytes).
cudaError_t launch_merkle(uint32_t* nodes, int layers, int hash_kind, cudaStream_t s, int tile_log = 0,
                          const MailSlot& mail = MailSlot());
extern int merkle_tile_log;

// count messages of `size` bytes (size % 4 == 0) -> count digests.
cudaError_t launch_hash_many(const uint8_t* in, size_t size, size_t count, uint8_t* out, int hash_kind,
                             cudaStream_t s);

// Searches nonces [start, start + count) and atomically lowers *best to any nonce whose digest's
// first 8 bytes (LE) are <= threshold (proof_of_work.rs:68-166). best[1] must be zero: it counts
// finished CTAs, and when mail.data is set the last one publishes best[0] (8 bytes) there.
cudaError_t launch_pow(const uint32_t challenge[8], uint64_t threshold, uint64_t start, uint64_t count,
                       unsigned long long* best, int hash_kind, cudaStream_t s, const MailSlot& mail = MailSlot());

// out[i*cols .. (i+1)*cols) = matrix[idx[i]*cols ..]
template <class F>
cudaError_t launch_gather_rows(const F* matrix, size_t cols, const uint64_t* idx, size_t n, F* out, cudaStream_t s);
// Authentication paths with repeats: out[((j layers + l) 8 + w)] = word w of the sibling at layer l
// (leaves: l = 0) of the ancestor of leaf idx[j], i.e. node (2^(layers+1) - 2^(layers+1-l)) +
// ((idx[j] >> l) ^ 1) of the node array; the host picks the reference's deduplicated node order
// out of these q x layers digests.
cudaError_t launch_gather_paths(const uint32_t* nodes, const uint64_t* idx, size_t q, int layers, uint32_t* out,
                                cudaStream_t s);

// ---------------------------------------------------------------------------------------------
// Sumcheck-side kernels (reference algebra/sumcheck.rs, multilinear.rs, algebra/mod.rs)
// ---------------------------------------------------------------------------------------------
// Number of partial (c0, c2) pairs written by the reduce kernels for a vector of n elements.
size_t sumcheck_partials(size_t n);

// The (c0, c2) kernels below write one partial pair per block. When `counter` is non-null (two
// zeroed u32 on the device: arrival count, launch sequence) the last block also sums the partials
// into out[0..2), re-zeroes the arrival count and publishes the pair: it increments the sequence
// and stores it as a u32 right after out[1] (out needs room for it) once the values are visible
// system-wide, so `out` can be host-mapped memory that the host polls.
// (c0, c2) of vectors a, b of n = 2^k elements -> partials (2 elements per block)
template <class T>
cudaError_t launch_sumcheck_compute(const T* a, const T* b, size_t n, T* partials, size_t* nparts, cudaStream_t s,
                                    T* out = nullptr, unsigned int* counter = nullptr);
// Folds a, b (n elements) with weight r in place to n/2 and computes (c0, c2) of the result.
template <class T>
cudaError_t launch_fold_compute(T* a, T* b, size_t n, T r, T* partials, size_t* nparts, cudaStream_t s,
                                T* out = nullptr, unsigned int* counter = nullptr);
// v[i] += (v[i + n/2] - v[i]) * r for i < n/2
template <class T>
cudaError_t launch_fold(T* v, size_t n, T r, cudaStream_t s);
// The same fold of two vectors of length n in one launch (the end of a sumcheck: a and b).
template <class T>
cudaError_t launch_fold2(T* v, T* w, size_t n, T r, cudaStream_t s);
// Sums nparts (c0, c2) partials into out[0..2).
template <class T>
cudaError_t launch_reduce_pairs(const T* partials, size_t nparts, T* out, cudaStream_t s);

// acc[i] += scalar * eq(point, i), point[0] is the most significant index bit (multilinear.rs:170-190).
// tables: scratch of 2^ceil(nv/2) + 2^floor(nv/2) elements; point is a device array.
template <class T>
cudaError_t launch_eval_eq(T* acc, const T* point, int nv, T scalar, T* tables, cudaStream_t s);

// acc[i] += sum_j scalars[j] * points[j]^i for i < n (algebra/mod.rs:154-177). Device arrays.
template <class T>
cudaError_t launch_geometric_accumulate(T* acc, size_t n, const T* scalars, const T* points, size_t m,
                                        cudaStream_t s);

// acc[i] += sum_j scalars[j] * w_N^(exps[j] * i) for i < n, points given as exponents of the
// N-th root of unity (in-domain evaluation points). Device arrays; N = 2^logN.
// Up to 4096 entries the (entry, query) pairs are also split over the queries: inside a CTA over
// 2^te_log entries, and across `groups` CTAs per tile of entries (the late rounds' covectors:
// 24 -> 5-9 us). Larger covectors keep one CTA thread per entry over all queries, where the
// root-table gathers are bound by L2 sector traffic either way. With groups > 1 the CTAs
// write partial sums (partials: groups * n elements) and the last CTA of a tile adds them (counters:
// GR_MAX_TILES words, zero before the first launch, re-armed by the kernel). Without scratch the
// launch uses one group.
static constexpr int GR_MAX_TILES = 4096;
struct GeometricSplit {
  bool split;  // false: one entry per thread (or several) over all queries
  int te_log;  // entries per CTA = 2^te_log (CTA threads / 2^te_log query subgroups)
  int groups;  // query groups across CTAs per tile of entries
};
inline GeometricSplit geometric_split_plan(size_t n, size_t m, bool scratch) {
  GeometricSplit p{false, 8, 1};
  if (n == 0 || m == 0 || n > 4096) return p;
  p.split = true;
  int te = 0;
  while (te < 8 && ((size_t)1 << te) < n) ++te;
  p.te_log = te;
  const size_t tiles = (n + ((size_t)1 << te) - 1) >> te, sub = (size_t)256 >> te;
  if (scratch && tiles <= (size_t)GR_MAX_TILES) {
    // about four waves of CTAs, at least eight queries per (CTA, subgroup)
    size_t g = (608 + tiles - 1) / tiles;
    g = std::min(g, std::max<size_t>(1, m / (8 * sub)));
    p.groups = (int)std::max<size_t>(1, std::min<size_t>(g, 64));
  }
  return p;
}
template <class T>
cudaError_t launch_geometric_roots(T* acc, size_t n, const T* scalars, const uint64_t* exps, size_t m, int logN,
                                   RootTab rt, cudaStream_t s, T* partials = nullptr,
                                   unsigned int* counters = nullptr);
// dense[e_k] = vals[k] for k < m (dense must be zeroed first; exponents distinct).
template <class T>
cudaError_t launch_scatter(T* dense, const uint64_t* idx, const T* vals, size_t m, cudaStream_t s);
// acc[i] += src[i] for i < n
template <class T>
cudaError_t launch_add(T* acc, const T* src, size_t n, cudaStream_t s);

// First two rounds of the initial sumcheck without materialising the lifted vector a = map(x) or
// the covector b = sum_l eq(point_l, .) * rlc_l (tables: per form, hi (2^h) then lo (2^l) entries,
// h = nv/2, l = nv - h, scalar folded into hi).
template <class T, class S>
cudaError_t launch_first_compute_eq(const S* x, size_t n, const T* tables, int nforms, int nv, T* partials,
                                    size_t* nparts, cudaStream_t s, T* out = nullptr, unsigned int* counter = nullptr);
// Folds map(x) and the eq covector with r (n -> n/2) into a_out / b_out and computes (c0, c2).
template <class T, class S>
cudaError_t launch_first_fold_compute_eq(const S* x, size_t n, T r, const T* tables, int nforms, int nv, T* a_out,
                                         T* b_out, T* partials, size_t* nparts, cudaStream_t s, T* out = nullptr,
                                         unsigned int* counter = nullptr);
// Row-factored rounds of the fused initial sumcheck (n = 2^nv, h = nv/2, l = nv - h): the covector
// is sum_f lo_f[j] F_f[H] at index H 2^l + j, with row factors F (2^rlog rows, per-form stride
// fstride; the hi tables at first). Folds a_in (length m = 2^(rlog + l)) with r into a_out (m/2; may
// be a_in), folds F into F_next (per-form stride 2^h), and computes (c0, c2) of the folded pair.
template <class T, class S>
cudaError_t launch_rows_fold_compute(const S* a_in, size_t m, T r, const T* F, size_t fstride, int rlog,
                                     const T* tables, int nforms, int nv, T* a_out, T* F_next, T* partials,
                                     size_t* nparts, cudaStream_t s, T* out = nullptr, unsigned int* counter = nullptr);
// Folds a (length m) with r in place and writes the folded covector (m/2 values) from row factors F.
template <class T>
cudaError_t launch_rows_finish(T* a, size_t m, T r, const T* F, int rlog, const T* tables, int nforms, int nv,
                               T* b_out, cudaStream_t s);
// sum_i map(x_i) * eq(point, i) for n <= 2^nv (implicit zero padding), from one eq table pair
// (hi: 2^(nv/2) entries, then lo: 2^(nv - nv/2)); block sums -> partials (reduce_singles).
template <class T, class S>
cudaError_t launch_mle_dot(const S* x, size_t n, const T* tables, int nv, T* partials, size_t* nparts,
                           cudaStream_t s);
// Builds the eq table of `cnt` coordinates point[off..off+cnt) scaled by scalar (device arrays).
template <class T>
cudaError_t launch_eq_table(const T* point, int off, int cnt, T scalar, T* table, cudaStream_t s);

// Initial sumcheck over a = sum_j c_j lift(x_j) and a covector that is a sum of tensor-product
// forms (eq forms of evaluation points, geometric forms of out-of-domain points): one pass over the
// vectors gives the 2^k sums from which the host derives all k round messages (launch_tensor_sums),
// a second pass after the last challenge writes the folded a and b (launch_tensor_fold). The
// tables hold, per form, the tensor weights of variables k..n-1 split into rows then columns
// (built by launch_tensor_tables from per-variable (alpha, beta) pairs).
static constexpr int TS_THREADS = 256;
static constexpr int TS_MAX_FORMS = 4;
static constexpr int TS_MAX_RPC = 32;  // rows per CTA in the sums pass

struct TensorShape {
  int k, R, C;          // folded variables, row bits, column bits (n = k + R + C)
  int nvec, nforms;     // vectors (RLC'd) and tensor forms
  uint64_t vec_stride;  // elements between consecutive vectors
  int rpc;              // rows per CTA (sums pass)
  int cpt;              // adjacent columns per thread (sums pass; 2 for 8-byte source elements)
  int threads;          // CTA threads (sums pass; a multiple of 32)
  uint64_t col_tiles, row_groups;
  uint64_t grid() const { return ((uint64_t)nvec << k) * row_groups * col_tiles; }
};

// src_bytes / src_aligned16: source element size and whether the vectors start on a 16-byte boundary
// (two 8-byte columns per thread are read with one 16-byte load).
inline TensorShape tensor_plan(int nvars, int k, int nvec, int nforms, uint64_t vec_stride, size_t src_bytes,
                               bool src_aligned16) {
  TensorShape sh;
  sh.k = k;
  const int rest = nvars - k;
  sh.R = std::min(rest, std::max(4, rest - 12));
  sh.C = rest - sh.R;
  sh.nvec = nvec;
  sh.nforms = nforms;
  sh.vec_stride = vec_stride;
  sh.rpc = (int)std::min<uint64_t>(1ull << sh.R, TS_MAX_RPC);
  const uint64_t cols = 1ull << sh.C;
  sh.cpt = (src_bytes == 8 && src_aligned16 && cols >= 64 && vec_stride % 2 == 0) ? 2 : 1;
  sh.threads = (int)std::max<uint64_t>(32, std::min<uint64_t>(TS_THREADS, cols / sh.cpt));
  sh.col_tiles = (cols / sh.cpt + sh.threads - 1) / sh.threads;
  sh.row_groups = (1ull << sh.R) / sh.rpc;
  return sh;
}

template <class T, class S>
cudaError_t launch_tensor_sums(const S* x, const TensorShape& sh, const T* tables, T* partials, T* out,
                               unsigned int* counter, cudaStream_t s,
                               const MailSlot& mail = MailSlot());
template <class T, class S>
cudaError_t launch_tensor_fold(const S* x, const TensorShape& sh, const T* w, const T* kf, const T* tables, T* a_out,
                               T* b_out, unsigned int* err, cudaStream_t s);
// Every form's row table (2^R) and column table (2^C) in one launch, from 2 (R + C) (alpha, beta)
// values per form; out holds nforms x (2^R + 2^C) entries, form-major, rows first, entry e of a
// table over cnt variables being prod_q (bit_{cnt-1-q}(e) ? beta_q : alpha_q).
template <class T>
cudaError_t launch_tensor_tables(const T* ab, int nforms, int R, int C, T* out, cudaStream_t s);

// dst[i] = map(v0[i]) + sum_{j>=1} coeffs[j] * v_j[i]  (lift + mixed_scalar_mul_add, algebra/mod.rs:51-98)
template <class T, class S>
cudaError_t launch_lift_rlc(T* dst, const S* const* vecs, const T* coeffs, size_t nvec, size_t n, cudaStream_t s);

// sum_i coeffs[i] x^i (mixed_univariate_evaluate, algebra/mod.rs:105-129) -> partials; reduce with
// launch_reduce_singles.
template <class T, class S>
cudaError_t launch_univariate_eval(const S* coeffs, size_t n, T x, T* partials, size_t* nparts, cudaStream_t s);
template <class T>
cudaError_t launch_reduce_singles(const T* partials, size_t nparts, T* out, cudaStream_t s);

}  // namespace whir
