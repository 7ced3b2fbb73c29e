// Perturbed wavefunctions and linear response (ccpert.cc, ccresp.cc), plus named
// tensor access for the C ABI.
#pragma once

#include <string>

#include "cc.h"

namespace ucc {

struct Perturbation {
  int id = 0;
  double omega = 0.0;
  std::string pfx;  // prefix of this perturbation's arrays in the context store
  bool right_done = false, left_done = false;
};

int pert_create(Ctx& c, const double* pert, double omega);
CCSDResult pert_solve(Ctx& c, int handle, bool right);
double linresp(Ctx& c, int hx, int hy);

Tensor named_tensor(Ctx& c, const std::string& name);
void set_named_tensor(Ctx& c, const std::string& name, const double* host, size_t count);

}  // namespace ucc
