/* ORACLE — test infrastructure only. C API of the CPU restatement (loaded by tests/ and by the
 * CPU-baseline leg of bench.py through ctypes). Field elements are canonical little-endian u64
 * limbs; extension elements are their base coefficients in increasing degree. */
#ifndef WHIR_ORACLE_API_H
#define WHIR_ORACLE_API_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Embedding / field ids, matching src/bin/main.rs's AvailableFields dispatch:
 * Goldilocks1 = Identity<Field64>, Goldilocks2 = Basefield<Field64_2>,
 * Goldilocks3 = Basefield<Field64_3>, Field192 / Field256 = Identity<F>. */
enum {
  ORACLE_GOLDILOCKS1 = 0,
  ORACLE_GOLDILOCKS2 = 1,
  ORACLE_GOLDILOCKS3 = 2,
  ORACLE_FIELD192 = 4,
  ORACLE_FIELD256 = 5
};

typedef struct oracle_protocol_params {
  int32_t unique_decoding;
  uint64_t starting_log_inv_rate;
  uint64_t initial_folding_factor;
  uint64_t folding_factor;
  uint64_t security_level;
  uint64_t pow_bits;
  uint64_t batch_size;
  uint8_t hash_id[32];
} oracle_protocol_params;

typedef struct oracle_proof oracle_proof;

const char* oracle_last_error(void);
int oracle_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
