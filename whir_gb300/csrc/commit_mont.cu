// Encode, gather and canonical-conversion kernels instantiated for the multi-limb Montgomery fields
// Field192 and Field256 (kept in their own translation unit so it compiles in parallel).
#include "encode.cuh"

namespace whir {

WHIR_ENCODE_INST(F192)
WHIR_ENCODE_INST(F256)

}  // namespace whir
