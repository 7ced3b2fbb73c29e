// Mixed-precision (BF16 hi+lo split, FP32 accumulate) tensor-core path.  Until the
// tcgen05 kernels are enabled every entry point declines and the caller runs FP64.
#include "core.h"

namespace ucc {

bool mixed_gemm(Ctx&, int64_t, int64_t, int64_t, double, const double*, int64_t, int64_t, const double*, int64_t,
                int64_t, double, double*, int64_t, int64_t) {
  return false;
}

bool mixed_triples_prepare(Ctx&) { return false; }
bool mixed_triples_batch(Ctx&, int, const int*, double*) { return false; }

}  // namespace ucc
