// Sumcheck-side kernels instantiated for the multi-limb Montgomery fields Field192 and Field256
// (identity embedding: coefficient vectors and statements over the same field).
#include "sumcheck.cuh"

namespace whir {

WHIR_SC_INST(F192)
WHIR_SC_INST(F256)
WHIR_SC_EMBED_INST(F192, F192)
WHIR_SC_EMBED_INST(F256, F256)

}  // namespace whir
