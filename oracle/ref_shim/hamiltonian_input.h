// Synthetic Hamiltonian file reader shared by the reference harness (test
// infrastructure).  File layout is documented in ugacc_gb300/generator.py.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace psi {
namespace ugacc {

struct HamiltonianInput {
  int no = 0, nv = 0, naux = 0, nact = 0, npert = 0;
  std::vector<double> eps;                 // [nact]
  std::vector<std::vector<double>> perts;  // npert x [nact*nact]
  std::vector<double> ints;                // [nact^4] <pq|rs>
};

inline HamiltonianInput& current_input() {
  static HamiltonianInput in;
  return in;
}

inline void load_input(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  auto rd = [&](void* p, size_t bytes) {
    if (bytes && std::fread(p, 1, bytes, f) != bytes) throw std::runtime_error("short read in " + path);
  };
  char magic[4];
  rd(magic, 4);
  if (std::string(magic, 4) != "UGAH") throw std::runtime_error("bad magic in " + path);
  int32_t hdr[6];
  rd(hdr, sizeof(hdr));
  if (hdr[0] != 1) throw std::runtime_error("unsupported file version");
  HamiltonianInput& in = current_input();
  in.no = hdr[1];
  in.nv = hdr[2];
  in.naux = hdr[3];
  in.npert = hdr[4];
  const int has_ints = hdr[5];
  in.nact = in.no + in.nv;
  const size_t n = (size_t)in.nact;
  in.eps.resize(n);
  rd(in.eps.data(), n * sizeof(double));
  // skip the three-index factors: the reference works from the 4-index integrals
  if (std::fseek(f, (long)(sizeof(double) * (size_t)in.naux * n * n), SEEK_CUR) != 0)
    throw std::runtime_error("seek failed");
  in.perts.assign(in.npert, std::vector<double>(n * n));
  for (int k = 0; k < in.npert; k++) rd(in.perts[k].data(), n * n * sizeof(double));
  if (!has_ints) throw std::runtime_error("input file carries no 4-index integrals");
  in.ints.resize(n * n * n * n);
  rd(in.ints.data(), in.ints.size() * sizeof(double));
  std::fclose(f);
}

}  // namespace ugacc
}  // namespace psi
