// ntk_refine_m32d.cu -- kernel instances of ntk_refine.cuh (one TU per M and carry mode, for parallel builds).
#include "ntk_refine.cuh"

namespace ntk {
template int refine_dispatch<32, true, 1>(const double*, double*, int, const Batch&, const RefineArgs&, bool, int,
                                          int, int, cudaStream_t);
}  // namespace ntk
