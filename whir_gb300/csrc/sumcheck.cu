// Sumcheck-side kernels instantiated for the Goldilocks family: the base field Goldilocks and its
// degree-2 and degree-3 extensions, with coefficient vectors over the base field.
#include "sumcheck.cuh"

namespace whir {

// Work items (quads of the fold-and-compute round) per thread, by size: four at n >= 2^20, where one
// per thread left the CTAs waiting at the reduction barriers and the last block summing 1024
// partials (fold-and-compute at 2^20: 45.0 us with one, 27.2 us with four); fewer below, where a
// small grid leaves the GPU idle (at 2^16: 15.6 us with one against 21.7 us with four).
size_t sumcheck_partials(size_t n) {
  const size_t items = n >= (1ull << 20) ? 4 : (n >= (1ull << 18) ? 2 : 1);
  size_t work = std::max<size_t>(n / 4, 1);
  return std::min(SC_MAX_BLOCKS, (work + SC_THREADS * items - 1) / (SC_THREADS * items));
}

WHIR_SC_INST(Gl)
WHIR_SC_INST(Gl2)
WHIR_SC_INST(Gl3)
WHIR_SC_EMBED_INST(Gl, Gl)
WHIR_SC_EMBED_INST(Gl2, Gl)
WHIR_SC_EMBED_INST(Gl3, Gl)
template cudaError_t launch_lift_rlc<Gl2, Gl2>(Gl2*, const Gl2* const*, const Gl2*, size_t, size_t, cudaStream_t);
template cudaError_t launch_lift_rlc<Gl3, Gl3>(Gl3*, const Gl3* const*, const Gl3*, size_t, size_t, cudaStream_t);
template cudaError_t launch_univariate_eval<Gl2, Gl2>(const Gl2*, size_t, Gl2, Gl2*, size_t*, cudaStream_t);
template cudaError_t launch_univariate_eval<Gl3, Gl3>(const Gl3*, size_t, Gl3, Gl3*, size_t*, cudaStream_t);
template cudaError_t launch_rows_fold_compute<Gl2, Gl2>(const Gl2*, size_t, Gl2, const Gl2*, size_t, int, const Gl2*,
                                                        int, int, Gl2*, Gl2*, Gl2*, size_t*, cudaStream_t, Gl2*,
                                                        unsigned int*);
template cudaError_t launch_rows_fold_compute<Gl3, Gl3>(const Gl3*, size_t, Gl3, const Gl3*, size_t, int, const Gl3*,
                                                        int, int, Gl3*, Gl3*, Gl3*, size_t*, cudaStream_t, Gl3*,
                                                        unsigned int*);

}  // namespace whir
