// Contraction engine: einsum-style two-operand contractions on device tensors.
#pragma once

#include <string>

#include "core.h"

namespace ucc {

// C[c] = alpha * sum A[a] B[b] + beta * C[c] for spec "a,b->c" (one letter per axis).
// Every output label must occur in exactly one input; summed labels occur in both.
// An index group that cannot be addressed with one stride is gathered into a dense
// scratch copy first; everything else is read in place by the strided GEMM.
void contract(Ctx& c, const std::string& spec, double alpha, const Tensor& A, const Tensor& B, double beta,
              const Tensor& C);

// C[c] = alpha * A[a] + beta * C[c] for spec "a->c" (a permutation of labels).
void transpose_add(Ctx& c, const std::string& spec, double alpha, const Tensor& A, double beta, const Tensor& C);

// View of T with axes relabelled: spec "abcd->cdab" returns T viewed with axes (c,d,a,b).
Tensor view(const Tensor& T, const std::string& spec);

// Full contraction sum A[a] B[a] (same labels, any layouts), result on the host.
double dot_all(Ctx& c, const Tensor& A, const Tensor& B);

// Dense scratch tensor (stream-ordered allocation freed when the holder dies).
struct Temp {
  Scratch buf;
  Tensor t;
  Temp(Ctx& c, const std::vector<int64_t>& dims, bool zero = false);
  operator Tensor&() { return t; }
  Tensor* operator->() { return &t; }
};

}  // namespace ucc
