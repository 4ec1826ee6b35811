/* whir_gb300 — C ABI of the GB300 (sm_103a) WHIR prover path.
 *
 * Each entry point replaces one interface of the reference crate (WizardOfMenlo/whir); the
 * citation beside it names the Rust item it stands in for. Conventions:
 *   - Every function returns 0 on success or a negative whir_status; none aborts the process.
 *     whir_last_error() describes the last failure on the calling thread.
 *   - Field elements are canonical little-endian u64 limbs (Goldilocks: 1 limb per base
 *     coefficient); extension elements list their base coefficients in increasing degree.
 *   - Pointers are host pointers unless a `flags` argument carries WHIR_DEVICE_PTRS, in which case
 *     the data pointers are device pointers on the context's device.
 *   - A whir_ctx owns a CUDA stream (all kernels and results), a second stream for uploading
 *     commit inputs from host memory while the encode runs, and a cache of device buffers in front
 *     of the stream-ordered memory pool; calls on one context must not overlap (serialise them per
 *     context); different contexts may be used from different threads.
 *   - There is no CPU fallback: without a usable CUDA device whir_ctx_create fails with
 *     WHIR_ERR_NO_DEVICE.
 */
#ifndef WHIR_GB300_H
#define WHIR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum whir_status {
  WHIR_OK = 0,
  WHIR_REJECT = 1,           /* verifier rejected (VerificationError) */
  WHIR_ERR_INVALID = -1,     /* bad argument: size mismatch, unknown id, non-canonical element */
  WHIR_ERR_UNSUPPORTED = -2, /* shape valid for the reference but not implemented on the device */
  WHIR_ERR_CUDA = -3,        /* CUDA runtime failure */
  WHIR_ERR_NO_DEVICE = -4,   /* no usable CUDA device */
  WHIR_ERR_POW = -5,         /* proof of work exhausted its search bound */
  WHIR_ERR_INTERNAL = -6
} whir_status;

/* Field / embedding ids, as src/bin/main.rs:84-103 dispatches AvailableFields:
 *   GOLDILOCKS1 = Identity<Field64>, GOLDILOCKS2 = Basefield<Field64_2>,
 *   GOLDILOCKS3 = Basefield<Field64_3> (src/algebra/fields.rs:85-143, embedding.rs:141-153). */
enum {
  WHIR_GOLDILOCKS1 = 0,
  WHIR_GOLDILOCKS2 = 1,
  WHIR_GOLDILOCKS3 = 2,
  WHIR_FIELD192 = 4,
  WHIR_FIELD256 = 5
};

#define WHIR_DEVICE_PTRS 1u

typedef struct whir_ctx whir_ctx;
typedef struct whir_config whir_config;
typedef struct whir_prover_state whir_prover_state;
typedef struct whir_witness whir_witness;

/* ProtocolParameters (src/parameters.rs:9-24). hash_id is the 32-byte EngineId
 * (src/engines.rs:22-23), e.g. Blake3 = 03e01749…5cc05b4c (src/hash/blake3_engine.rs:19). */
typedef struct whir_params {
  int32_t unique_decoding;
  uint64_t starting_log_inv_rate;
  uint64_t initial_folding_factor;
  uint64_t folding_factor;
  uint64_t security_level;
  uint64_t pow_bits;
  uint64_t batch_size;
  uint8_t hash_id[32];
} whir_params;

const char* whir_last_error(void);

/* ---- context -------------------------------------------------------------------------------- */
int whir_ctx_create(int device, whir_ctx** out);
/* A context whose streams have a raised scheduling priority (no reference counterpart): priority 0
 * is whir_ctx_create's; each step above raises it toward the device's greatest priority. A serving
 * loop proves its largest requests on such contexts so they are not slowed by the small ones. */
int whir_ctx_create_priority(int device, int priority, whir_ctx** out);
int whir_ctx_destroy(whir_ctx* ctx);
/* Blocks until all work queued on the context's stream has finished. */
int whir_ctx_synchronize(whir_ctx* ctx);
/* Instrumentation (no counterpart in the reference, which has no device):
 *   whir_ctx_launch_count   kernel launches issued by this library since the context was created
 *   whir_ctx_stream         the context's cudaStream_t (for CUDA-event timing by the caller)
 *   whir_ctx_transfer_bytes cumulative host->device / device->host bytes moved by the context
 *   whir_ctx_set_profiling  enable CUDA-event timing of kernel families (resets the counters)
 *   whir_ctx_profile        per-family milliseconds and call counts; returns the number of
 *                           families: 0 encode, 1 merkle, 2 sumcheck, 3 eq, 4 geometric, 5 lift,
 *                           6 pow, 7 gather, 8 univariate */
uint64_t whir_ctx_launch_count(const whir_ctx* ctx);
void* whir_ctx_stream(const whir_ctx* ctx);
int whir_ctx_transfer_bytes(const whir_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes);
int whir_ctx_set_profiling(whir_ctx* ctx, int enabled);
int whir_ctx_profile(whir_ctx* ctx, double* ms, uint64_t* calls, size_t n_families);
/* Device allocation helpers on the context's stream-ordered pool (for callers that keep inputs
 * resident in HBM between calls). */
int whir_device_alloc(whir_ctx* ctx, size_t bytes, void** out);
int whir_device_free(whir_ctx* ctx, void* ptr);
/* Page-locked host memory (cudaHostAlloc, usable from every context): inputs handed to whir_commit
 * / whir_prove from such buffers are copied by DMA at full link speed while the encode runs; from
 * ordinary (pageable) memory the copy is staged by the driver and runs several times slower. */
int whir_host_alloc(size_t bytes, void** out);
int whir_host_free(void* ptr);
int whir_memcpy_h2d(whir_ctx* ctx, void* dst, const void* src, size_t bytes);
int whir_memcpy_d2h(whir_ctx* ctx, void* dst, const void* src, size_t bytes);

/* ---- protocol: Config / ProverState / commit / prove ------------------------------------------- */
/* whir::Config::<M>::new(size, &params) (src/protocols/whir/config.rs:16-152). */
int whir_config_new(int field, const whir_params* params, uint64_t size, whir_config** out);
int whir_config_free(whir_config* cfg);
/* JSON summary of the derived round schedule (sizes, sample counts, PoW thresholds). */
int whir_config_json(const whir_config* cfg, char* buf, size_t cap);

/* ciborium::into_writer(&config): the CBOR of the serde form of whir::Config
 * (src/transcript/mod.rs:111-121, src/protocols/whir/mod.rs:29-46), whose SHA3-512 is the
 * protocol id. Writes up to cap bytes to buf (nullable) and the full length to *len. */
int whir_config_cbor(const whir_config* cfg, uint8_t* buf, size_t cap, size_t* len);
/* ProverState::new_std(&DomainSeparator::protocol(&config).session(&session).instance(&Empty))
 * (src/transcript/mod.rs:110-181). */
int whir_prover_state_new(const whir_config* cfg, const char* session, size_t session_len,
                          whir_prover_state** out);
int whir_prover_state_free(whir_prover_state* ps);
/* Proof { narg_string, hints } (src/transcript/mod.rs:63-70, 235-243); pointers stay valid until
 * the next call on the state. */
int whir_prover_state_proof(const whir_prover_state* ps, const uint8_t** narg, size_t* narg_len,
                            const uint8_t** hints, size_t* hints_len);

/* Config::commit(&mut prover_state, &[&[Source]]) -> Witness (src/protocols/whir/mod.rs:79-92,
 * irs_commit.rs:292-350). vectors: batch_size contiguous vectors of `size` source elements. The
 * witness (codeword matrix and Merkle nodes) stays resident on the device. */
int whir_commit(whir_ctx* ctx, const whir_config* cfg, whir_prover_state* ps, const uint64_t* vectors,
                uint32_t flags, whir_witness** out);
/* Config::commit for n independent jobs at once: the batched form of whir_commit (the reference
 * commits one job per call, irs_commit.rs:292-350). All jobs share one embedding and one hash
 * engine; their sizes may differ. The device work of every job runs in shared launches (one encode
 * column pass, one encode row pass with the leaf hashes, one Merkle launch per tile step, one
 * fetch of all roots); then each job's transcript receives its root and out-of-domain samples
 * exactly as whir_commit writes them. out[j] receives job j's witness (NULL on failure). */
int whir_commit_batch(whir_ctx* ctx, size_t n, const whir_config* const* cfgs, whir_prover_state* const* pss,
                      const uint64_t* const* vectors, uint32_t flags, whir_witness** out);
int whir_witness_free(whir_witness* w);
int whir_witness_root(const whir_witness* w, uint8_t root[32]);

/* Config::prove (src/protocols/whir/prover.rs:50-315).
 *   vectors:     n_witnesses * batch_size contiguous vectors (same order as the witnesses)
 *   mle_points:  n_points points of log2(size) target elements (MultilinearExtension forms)
 *   covectors:   n_covectors explicit covectors of `size` target elements (Covector forms,
 *                ordered after the MLE forms)
 *   evaluations: (n_points + n_covectors) x n_vectors target elements, row-major
 *   eval_point_out (nullable): receives FinalClaim.evaluation_point (log2(size) elements)
 *   rlc_out (nullable): receives FinalClaim.rlc_coefficients (n_points + n_covectors elements) */
int whir_prove(whir_ctx* ctx, const whir_config* cfg, whir_prover_state* ps, const uint64_t* vectors,
               uint32_t flags, whir_witness* const* witnesses, size_t n_witnesses, const uint64_t* mle_points,
               size_t n_points, const uint64_t* covectors, size_t n_covectors, const uint64_t* evaluations,
               uint64_t* eval_point_out, uint64_t* rlc_out);

/* Config::verify (src/protocols/whir/verifier.rs:45-265) followed by FinalClaim::verify
 * (src/protocols/whir/mod.rs:63-74) against the statement, on the host (no device needed).
 *   session:       the session string the prover state was created with
 *   narg / hints:  the proof (whir_prover_state_proof)
 *   n_commitments: number of witnesses the prover committed (each batch_size vectors)
 *   mle_points, covectors, evaluations: the statement, laid out as for whir_prove
 * Returns WHIR_OK when the proof is accepted, WHIR_REJECT when a check fails (the reason is in
 * whir_verify_last_reason()), or a negative status for bad arguments. */
int whir_verify(const whir_config* cfg, const char* session, size_t session_len, const uint8_t* narg,
                size_t narg_len, const uint8_t* hints, size_t hints_len, size_t n_commitments,
                const uint64_t* mle_points, size_t n_points, const uint64_t* covectors, size_t n_covectors,
                const uint64_t* evaluations);
/* Reason of the calling thread's last whir_verify rejection or error (no reference counterpart). */
const char* whir_verify_last_reason(void);

/* ---- autotuning (no reference counterpart: the reference has no device schedules) -------------
 * whir_autotune times, on this context's device, every valid encode plan (whole cosets per CTA, or
 * the four-step split's row-pass size and column-pass width) and Merkle tile height for the
 * commitment shapes that Config::new derived for `cfg` (the initial commitment and every round's),
 * and records the fastest in a process-wide table that later encodes and trees of those shapes use
 * (results are bit-identical whatever the choice). report (nullable) receives a JSON summary of the
 * candidates' milliseconds. The table is exported / imported as text lines
 *   "encode <n_msgs> <msg_len> <codeword_len> <elem_bytes> <mode> <logC2> <W> <G>"
 *   "merkle <layers> <tile_log>"
 * so a serving process can load choices measured earlier; whir_autotune_clear empties it. */
int whir_autotune(whir_ctx* ctx, const whir_config* cfg, int reps, char* report, size_t cap);
int whir_autotune_export(char* buf, size_t cap, size_t* len);
int whir_autotune_import(const char* text);
int whir_autotune_clear(void);

/* ---- operator-level entry points --------------------------------------------------------------- */
/* ReedSolomon::interleaved_encode (src/algebra/ntt/mod.rs:89-99, cooley_tukey.rs:411-477) via
 * ntt::interleaved_rs_encode (ntt/mod.rs:120-128). msgs: n_msgs x msg_len (message-major); out:
 * codeword_len x n_msgs (row-major). masks: n_msgs x mask_len (may be NULL when mask_len == 0);
 * message m is encoded as its msg_len coefficients followed by its mask_len mask values. */
int whir_rs_interleaved_encode(whir_ctx* ctx, int field, const uint64_t* msgs, size_t n_msgs, size_t msg_len,
                               const uint64_t* masks, size_t mask_len, size_t codeword_len, uint64_t* out,
                               uint32_t flags);
/* ReedSolomon::evaluation_points (ntt/mod.rs:82-87, cooley_tukey.rs:375-402); host computation. */
int whir_rs_evaluation_points(int field, size_t masked_len, size_t codeword_len, const uint64_t* indices, size_t n,
                              uint64_t* out);
/* HashEngine::hash_many (src/hash/mod.rs:79-85) for the engine with this EngineId. */
int whir_hash_many(whir_ctx* ctx, const uint8_t engine_id[32], size_t size, const uint8_t* in, size_t count,
                   uint8_t* out, uint32_t flags);
/* merkle_tree::Config::commit layer hashing (src/protocols/merkle_tree.rs:82-127): leaves (n
 * digests) -> all 2^(L+1)-1 nodes, leaves zero-padded to 2^L, root last. */
int whir_merkle_nodes(whir_ctx* ctx, const uint8_t engine_id[32], const uint8_t* leaves, size_t n_leaves,
                      uint8_t* nodes_out, uint32_t flags);
/* compute_sumcheck_polynomial (src/algebra/sumcheck.rs:12-63) for power-of-two n. */
int whir_sumcheck_polynomial(whir_ctx* ctx, int field, const uint64_t* a, const uint64_t* b, size_t n, uint64_t* c0,
                             uint64_t* c2, uint32_t flags);
/* fold (src/algebra/sumcheck.rs:69-104) in place for power-of-two n; v keeps n/2 elements. */
int whir_fold(whir_ctx* ctx, int field, uint64_t* v, size_t n, const uint64_t* weight, uint32_t flags);
/* eval_eq (src/algebra/multilinear.rs:170-190): acc (2^nvars) += scalar * eq(point, .). */
int whir_eval_eq(whir_ctx* ctx, int field, uint64_t* acc, const uint64_t* point, size_t nvars,
                 const uint64_t* scalar, uint32_t flags);
/* geometric_accumulate (src/algebra/mod.rs:154-177): acc[i] += sum_j scalars[j] * points[j]^i. */
int whir_geometric_accumulate(whir_ctx* ctx, int field, uint64_t* acc, size_t n, const uint64_t* scalars,
                              const uint64_t* points, size_t m, uint32_t flags);
/* mixed_univariate_evaluate (src/algebra/mod.rs:105-129) for the embedding `field`. */
int whir_univariate_evaluate(whir_ctx* ctx, int field, const uint64_t* coeffs, size_t n, const uint64_t* point,
                             uint64_t* out, uint32_t flags);
/* lift (src/algebra/mod.rs:51-59): dst[i] = embedding.map(src[i]) for the embedding `field`
 * (n source elements in, n target elements out; Goldilocks2/3 put the value in the constant
 * coefficient). */
int whir_lift(whir_ctx* ctx, int field, const uint64_t* src, size_t n, uint64_t* dst, uint32_t flags);
/* Evaluation of the multilinear extension of n <= 2^nvars source values (implicitly zero-padded)
 * at a target-field point: MultilinearExtension's Evaluate (linear_form/multilinear_extension.rs:
 * 53-57 -> mixed_multilinear_extend, src/algebra/multilinear.rs:15-151). This is how callers compute
 * the `evaluations` a statement passes to whir_prove. */
int whir_multilinear_evaluate(whir_ctx* ctx, int field, const uint64_t* coeffs, size_t n, const uint64_t* point,
                              size_t nvars, uint64_t* out, uint32_t flags);
/* proof_of_work::Config::prove grinding (src/protocols/proof_of_work.rs:68-166): lowest nonce with
 * LE-u64(H(challenge || nonce_le || 0^24)[0..8]) <= threshold. */
int whir_pow_grind(whir_ctx* ctx, const uint8_t engine_id[32], const uint8_t challenge[32], uint64_t threshold,
                   uint64_t* nonce);

/* ---- no-allocation variant ---------------------------------------------------------------------
 * No counterpart in the reference. eval_eq (acc += scalar * eq(point, .)) for callers that cannot
 * call cudaMalloc where they need it: hosts that embed the prover behind an allocator they do not
 * control, callers with a fixed device-memory budget or that must not allocate at the call site. It
 * needs no whir_ctx and allocates nothing: acc_dev (2^nvars elements) and point_dev (nvars
 * elements) are caller-owned device buffers on the current device, scalar is one host element,
 * stream is a cudaStream_t (NULL = legacy default stream); the work is only enqueued.
 *   - Scratch: the two eq tables live in one file-scope device array of
 *     whir_eval_eq_noalloc_max_scratch() bytes (256 KiB), held on every device that loads the
 *     library until the process exits; nvars is limited to what fits,
 *     (2^ceil(nvars/2) + 2^floor(nvars/2)) * element bytes <= 256 KiB: nvars <= 28 for Goldilocks1,
 *     <= 26 for Goldilocks2, <= 24 for Goldilocks3. Larger nvars (or nvars == 0) is rejected with
 *     WHIR_ERR_INVALID.
 *   - Each call looks up the array's device address on the current device (cudaGetSymbolAddress),
 *     except while `stream` reports an active capture (cudaStreamIsCapturing), when it reuses the
 *     address found by the last call on that device that did look it up.
 *   - All calls share the array and it keeps the last call's tables; every call rewrites the
 *     tables before reading them. Calls whose work overlaps on the GPU (different streams, or
 *     different host threads on the same device) race on the array: serialise them.
 * Errors are reported through whir_noalloc_last_error(). */
int whir_eval_eq_noalloc(int field, uint64_t* acc_dev, const uint64_t* point_dev, size_t nvars,
                         const uint64_t* scalar, void* stream);
size_t whir_eval_eq_noalloc_max_scratch(void);
const char* whir_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* WHIR_GB300_H */
