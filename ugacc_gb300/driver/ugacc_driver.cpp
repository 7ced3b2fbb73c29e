// Command-line driver: the reference plugin's pipeline (ugacc.cc:108-241) on the
// C++ class surface of the GB300 library, for a Hamiltonian stored in the synthetic
// input format of ugacc_gb300/generator.py (three-index factors are used) or in an
// MO-integral file in the FCIDUMP layout (first non-blank text "&FCI"; NFZC / NFZV frozen
// core and virtual orbitals, hamiltonian.cc:24-27).
//
// usage: ugacc_driver <input.bin | FCIDUMP> [WFN=CCSD|CCSD_T] [DERTYPE=NONE|FIRST|SECOND]
//        [MAXITER=100] [R_CONVERGENCE=1e-7] [DIIS=1] [MY_OMEGA=0] [MYHAND=RIGHT|LEFT]
//        [PRECISION=FP64|MIXED] [REFINE_SWEEPS=2] [PRINT=0] [OOC=0|1] [NFZC=0] [NFZV=0]
// Prints one JSON object with the energies (and polarizabilities for DERTYPE=SECOND with
// the synthetic format's perturbations).
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include "../../include/ugacc_gb300.hpp"

using namespace ugacc_gb300;

namespace {
struct Input {
  int no = 0, nv = 0, naux = 0, npert = 0;
  std::vector<double> eps, B;
  std::vector<std::vector<double>> perts;
};

// true when the file's first non-blank characters are "&FCI" (any case)
bool is_fcidump(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[256];
  const size_t n = std::fread(buf, 1, sizeof buf, f);
  std::fclose(f);
  size_t k = 0;
  while (k < n && (buf[k] == ' ' || buf[k] == '\t' || buf[k] == '\r' || buf[k] == '\n')) k++;
  if (k + 4 > n || buf[k] != '&') return false;
  for (int j = 1; j < 4; j++)
    if (std::toupper((unsigned char)buf[k + j]) != "&FCI"[j]) return false;
  return true;
}

Input read_input(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  auto rd = [&](void* p, size_t n) {
    if (n && std::fread(p, 1, n, f) != n) throw std::runtime_error("short read");
  };
  char magic[4];
  rd(magic, 4);
  if (std::string(magic, 4) != "UGAH") throw std::runtime_error("not a synthetic Hamiltonian file");
  int32_t h[6];
  rd(h, sizeof h);
  Input in;
  in.no = h[1];
  in.nv = h[2];
  in.naux = h[3];
  in.npert = h[4];
  const size_t n = (size_t)in.no + in.nv;
  in.eps.resize(n);
  rd(in.eps.data(), n * 8);
  in.B.resize((size_t)in.naux * n * n);
  rd(in.B.data(), in.B.size() * 8);
  in.perts.assign(in.npert, std::vector<double>(n * n));
  for (auto& p : in.perts) rd(p.data(), p.size() * 8);
  std::fclose(f);
  return in;
}
}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s input.bin [KEY=VALUE ...]\n", argv[0]);
    return 2;
  }
  std::map<std::string, std::string> kv;
  for (int k = 2; k < argc; k++) {
    std::string a = argv[k];
    auto eq = a.find('=');
    if (eq != std::string::npos) kv[a.substr(0, eq)] = a.substr(eq + 1);
  }
  auto get = [&](const char* k, const char* d) { return kv.count(k) ? kv[k] : std::string(d); };
  try {
    const bool dump = is_fcidump(argv[1]);
    Input in;
    if (!dump) in = read_input(argv[1]);
    Options o;
    o.wfn = get("WFN", "CCSD");
    o.dertype = get("DERTYPE", "NONE");
    o.myhand = get("MYHAND", "RIGHT");
    o.precision = get("PRECISION", "FP64");
    o.maxiter = std::atoi(get("MAXITER", "100").c_str());
    o.refine_sweeps = std::atoi(get("REFINE_SWEEPS", "2").c_str());
    o.print = std::atoi(get("PRINT", "0").c_str());
    o.r_convergence = std::atof(get("R_CONVERGENCE", "1e-7").c_str());
    o.my_omega = std::atof(get("MY_OMEGA", "0").c_str());
    o.diis = get("DIIS", "1") == "1";
    o.ooc = get("OOC", "0") == "1";

    std::shared_ptr<Hamiltonian> H;
    if (dump) {
      H = Hamiltonian::from_fcidump(argv[1], std::atoi(get("NFZC", "0").c_str()), std::atoi(get("NFZV", "0").c_str()));
    } else {
      const int n = in.no + in.nv;
      std::vector<double> fock((size_t)n * n, 0.0);
      for (int p = 0; p < n; p++) fock[(size_t)p * n + p] = in.eps[p];
      H = std::make_shared<Hamiltonian>(in.no, in.nv, in.naux, fock.data(), in.B.data());
    }
    // the reference's CCWfn takes the SCF wavefunction first (ccwfn.h:14); here it is the
    // file's SCF energy (FCIDUMP input) or nothing (synthetic input)
    struct ScfReference {
      double energy;
    };
    auto ref = std::make_shared<ScfReference>(ScfReference{dump ? H->escf() : 0.0});
    auto cc = std::make_shared<CCWfn>(ref, H, o);
    const double ecc = cc->compute_energy();
    std::printf("{\"e_ccsd\": %.17g, \"e_t\": %.17g, \"e_cc\": %.17g", cc->eccsd(), cc->et(), ecc);
    if (dump)
      std::printf(", \"e_scf\": %.17g, \"e_frozen_core\": %.17g, \"e_total\": %.17g", H->escf(), H->efzc(),
                  H->escf() + ecc);
    if (o.dertype != "NONE") {
      auto hbar = std::make_shared<HBAR>(H, cc);
      auto lam = std::make_shared<CCLambda>(cc, hbar);
      lam->compute_lambda();
      CCDensity dens(cc, lam);
      const double e1 = dens.onepdm(), e2 = dens.twopdm();
      std::printf(", \"pseudoenergy\": %.17g, \"e_onepdm\": %.17g, \"e_twopdm\": %.17g", lam->pseudoenergy(), e1, e2);
      if (o.dertype == "SECOND" && in.npert >= 3) {
        const char* cart = "XYZ";
        std::vector<std::shared_ptr<CCPert>> mu(3);
        const int n = in.no + in.nv;
        for (int x = 0; x < 3; x++) {
          // the reference hands CCPert its perturbation as row pointers (ccpert.h:19)
          std::vector<double*> rows(n);
          for (int r = 0; r < n; r++) rows[r] = in.perts[x].data() + (size_t)r * n;
          mu[x] = std::make_shared<CCPert>(rows.data(), o.my_omega, cc, hbar, lam);
          mu[x]->solve(right);
          if (o.myhand != "RIGHT") mu[x]->solve(left);
          std::printf(", \"pseudoresponse_%c\": %.17g", cart[x], mu[x]->pseudoresponse(right));
        }
        for (int p = 0; p < 3; p++)
          for (int q = 0; q <= p; q++) {
            double a;
            if (p == q) {  // one perturbation on both sides: the single-argument form (ccresp.h:13)
              CCResp r(mu[p]);
              a = r.linresp(mu[p], mu[p]);
            } else {
              CCResp r(mu[p], mu[q]);
              a = 0.5 * r.linresp(mu[p], mu[q]) + 0.5 * r.linresp(mu[q], mu[p]);
            }
            std::printf(", \"alpha_%c%c\": %.17g", cart[p], cart[q], a);
          }
      }
    }
    std::printf("}\n");
  } catch (const ConvergenceError& e) {
    std::fprintf(stderr, "ugacc_driver: %s\n", e.what());
    return 3;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ugacc_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
