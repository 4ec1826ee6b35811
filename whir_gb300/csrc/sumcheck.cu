// Sumcheck-side kernels instantiated for the Goldilocks family: the base field Goldilocks and its
// degree-2 and degree-3 extensions, with coefficient vectors over the base field.
#include "sumcheck.cuh"

namespace whir {

// Four work items (quads of the fold-and-compute round) per thread: with one item per thread the
// round kernels' CTAs spent most of their time in the block reduction's barriers (ncu at n = 2^20:
// 20 % issue-active, barrier stalls first).
static constexpr size_t SC_ITEMS_PER_THREAD = 4;
size_t sumcheck_partials(size_t n) {
  size_t work = std::max<size_t>(n / 4, 1);
  return std::min(SC_MAX_BLOCKS, (work + SC_THREADS * SC_ITEMS_PER_THREAD - 1) / (SC_THREADS * SC_ITEMS_PER_THREAD));
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
