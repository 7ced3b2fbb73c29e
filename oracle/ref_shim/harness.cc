// Driver for the reference's own CC classes on a synthetic Hamiltonian
// (test infrastructure: it produces the golden values that pin the oracle).
//
// It walks the same pipeline as the plugin entry ugacc.cc:108-241:
//   Hamiltonian -> CCWfn::compute_energy -> [(T)] -> HBAR -> CCLambda::compute_lambda
//   -> CCDensity::onepdm/twopdm -> CCPert::solve per axis -> CCResp::linresp
// with the one-electron perturbations taken from the input file instead of psi4's
// property integrals (CCPert accepts a raw double**, ccpert.h:19).
//
// usage: ugacc_ref <input.bin> <outdir> [KEY=VALUE ...]
//   WFN=CCSD  DERTYPE=NONE|FIRST|SECOND  MAXITER=100  R_CONVERGENCE=1e-10  DIIS=1
//   TRIPLES=none|ooc|tjl|incore|all   MY_OMEGA=0.0   MYHAND=RIGHT|LEFT   DUMP=0|1
// TRIPLES calls the reference's (T) routines after the CCSD solve, exactly where
// compute_energy calls them for WFN=CCSD_T (ccwfn.cc:237-245, after build_tstar).
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "hamiltonian_input.h"
#include "psi4_shim.h"

// The harness reads the classes' protected arrays to dump them; the layout of the
// classes does not depend on access specifiers.
#define protected public
#define private public
#include "ccdensity.h"
#include "cclambda.h"
#include "ccpert.h"
#include "ccresp.h"
#include "ccwfn.h"
#include "hamiltonian.h"
#include "hbar.h"
#undef protected
#undef private

using psi::Options;
using psi::Wavefunction;
namespace U = psi::ugacc;

namespace {

using clk = std::chrono::steady_clock;
double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

struct Out {
  std::string dir;
  bool dump = false;
  std::vector<std::string> json;  // "key": value fragments
  std::vector<std::string> tensors;

  void num(const std::string& k, double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    json.push_back("\"" + k + "\": " + buf);
  }
  void str(const std::string& k, const std::string& v) { json.push_back("\"" + k + "\": \"" + v + "\""); }

  void write(const std::string& name, const std::vector<int>& shape, const std::function<double(size_t)>& at) {
    if (!dump) return;
    size_t n = 1;
    for (int d : shape) n *= (size_t)d;
    std::vector<double> buf(n);
    for (size_t k = 0; k < n; k++) buf[k] = at(k);
    FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write tensor " + name);
    std::fwrite(buf.data(), sizeof(double), n, f);
    std::fclose(f);
    std::ostringstream s;
    s << "\"" << name << "\": [";
    for (size_t k = 0; k < shape.size(); k++) s << (k ? ", " : "") << shape[k];
    s << "]";
    tensors.push_back(s.str());
  }
  void mat(const std::string& name, double** A, int r, int c) {
    write(name, {r, c}, [&](size_t k) { return A[k / c][k % c]; });
  }
  void t4(const std::string& name, double**** A, int p, int q, int r, int s) {
    write(name, {p, q, r, s}, [&](size_t k) {
      const size_t l = k % s, kk = k / s, j = kk % r, k2 = kk / r, i = k2 % q, h = k2 / q;
      return A[h][i][j][l];
    });
  }
  void finish() {
    std::string path = dir + "/result.json";
    FILE* f = std::fopen(path.c_str(), "w");
    std::fprintf(f, "{\n");
    for (size_t k = 0; k < json.size(); k++) std::fprintf(f, "  %s,\n", json[k].c_str());
    std::fprintf(f, "  \"tensors\": {");
    for (size_t k = 0; k < tensors.size(); k++) std::fprintf(f, "%s%s", k ? ", " : "", tensors[k].c_str());
    std::fprintf(f, "}\n}\n");
    std::fclose(f);
  }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s input.bin outdir [KEY=VALUE ...]\n", argv[0]);
    return 2;
  }
  std::map<std::string, std::string> kv = {{"WFN", "CCSD"},     {"DERTYPE", "NONE"},    {"MAXITER", "100"},
                                           {"R_CONVERGENCE", "1e-10"}, {"DIIS", "1"},   {"TRIPLES", "none"},
                                           {"MY_OMEGA", "0.0"}, {"MYHAND", "RIGHT"},    {"DUMP", "0"},
                                           {"OOC", "1"}};
  for (int k = 3; k < argc; k++) {
    std::string a = argv[k];
    auto eq = a.find('=');
    if (eq == std::string::npos) {
      std::fprintf(stderr, "bad argument %s\n", argv[k]);
      return 2;
    }
    kv[a.substr(0, eq)] = a.substr(eq + 1);
  }
  Out out;
  out.dir = argv[2];
  out.dump = kv["DUMP"] == "1";
  mkdir(out.dir.c_str(), 0755);
  FILE* logf = std::fopen((out.dir + "/log.txt").c_str(), "w");
  psi::outfile->set_file(logf);

  try {
    auto t0 = clk::now();
    U::load_input(argv[1]);
    const U::HamiltonianInput& in = U::current_input();
    const int no = in.no, nv = in.nv, nact = in.nact;
    out.num("no", no);
    out.num("nv", nv);
    out.num("load_s", secs(t0, clk::now()));

    Options options;
    options.set_str("WFN", kv["WFN"]);
    options.set_str("DERTYPE", kv["DERTYPE"]);
    options.set_str("REFERENCE", "RHF");
    options.set_str("MYHAND", kv["MYHAND"]);
    options.set_int("MAXITER", std::atoi(kv["MAXITER"].c_str()));
    options.set_double("R_CONVERGENCE", std::atof(kv["R_CONVERGENCE"].c_str()));
    options.set_bool("DIIS", kv["DIIS"] == "1");
    options.set_bool("OOC", kv["OOC"] == "1");  // the plugin's default is false (ugacc.cc:67)
    options.set_double("MY_OMEGA", std::atof(kv["MY_OMEGA"].c_str()));

    auto ref = std::make_shared<Wavefunction>(options);
    ref->nirrep_ = 1;
    ref->nmo_ = nact;
    ref->nso_ = nact;
    ref->nfrzc_ = 0;
    ref->doccpi_ = psi::Dimension({no});
    ref->soccpi_ = psi::Dimension({0});
    ref->frzcpi_ = psi::Dimension({0});
    ref->frzvpi_ = psi::Dimension({0});
    ref->nmopi_ = psi::Dimension({nact});
    ref->energy_ = 0.0;  // correlation energies only; the synthetic model has no SCF energy
    ref->molecule_ = std::make_shared<psi::Molecule>();

    std::shared_ptr<psi::PSIO> psio = std::make_shared<psi::PSIO>();
    std::vector<std::shared_ptr<psi::MOSpace> > spaces = {psi::MOSpace::all};

    auto ta = clk::now();
    std::shared_ptr<U::Hamiltonian> H(new U::Hamiltonian(psio, ref, spaces));
    out.num("hamiltonian_s", secs(ta, clk::now()));

    ta = clk::now();
    std::shared_ptr<U::CCWfn> cc(new U::CCWfn(ref, H, options));
    const double ecc = cc->compute_energy();
    out.num("ccsd_s", secs(ta, clk::now()));
    out.num("e_ccsd", ecc);
    out.mat("t1", cc->t1_, no, nv);
    out.t4("t2", cc->t2_, no, no, nv, nv);
    if (kv["WFN"] == "CCSD_T" && kv["DERTYPE"] == "FIRST") {
      // (T) gradient pieces left by compute_energy's tgrad_ooc or tgrad (ccwfn.cc:252-255)
      out.mat("s1", cc->s1_, no, nv);
      out.t4("s2", cc->s2_, no, no, nv, nv);
      out.mat("DooT", cc->Doo_, no, no);
      out.mat("DvvT", cc->Dvv_, nv, nv);
      out.mat("DovT", cc->Dov_, no, nv);
      out.t4("GoovvT", cc->Goovv_, no, no, nv, nv);
      out.t4("GooovT", cc->Gooov_, no, no, no, nv);
      out.t4("GvvvoT", cc->Gvvvo_, nv, nv, nv, no);
    }

    const std::string trip = kv["TRIPLES"];
    if (trip == "ooc" || trip == "all") {
      ta = clk::now();
      out.num("e_t_ooc", cc->tcorr_ooc());
      out.num("t_ooc_s", secs(ta, clk::now()));
    }
    if (trip == "tjl" || trip == "all") {
      ta = clk::now();
      out.num("e_t_tjl", cc->tcorr_ooc_TJL());
      out.num("t_tjl_s", secs(ta, clk::now()));
    }
    if (trip == "incore" || trip == "all") {
      ta = clk::now();
      out.num("e_t_incore", cc->tcorr());
      out.num("t_incore_s", secs(ta, clk::now()));
    }

    if (kv["DERTYPE"] != "NONE") {
      ta = clk::now();
      std::shared_ptr<U::HBAR> hbar(new U::HBAR(H, cc));
      out.num("hbar_s", secs(ta, clk::now()));
      out.mat("Hov", hbar->Hov_, no, nv);
      out.mat("Hoo", hbar->Hoo_, no, no);
      out.mat("Hvv", hbar->Hvv_, nv, nv);
      out.t4("Hoooo", hbar->Hoooo_, no, no, no, no);
      out.t4("Hvvvv", hbar->Hvvvv_, nv, nv, nv, nv);
      out.t4("Hvovv", hbar->Hvovv_, nv, no, nv, nv);
      out.t4("Hooov", hbar->Hooov_, no, no, no, nv);
      out.t4("Hovvo", hbar->Hovvo_, no, nv, nv, no);
      out.t4("Hovov", hbar->Hovov_, no, nv, no, nv);
      out.t4("Hvvvo", hbar->Hvvvo_, nv, nv, nv, no);
      out.t4("Hovoo", hbar->Hovoo_, no, nv, no, no);

      ta = clk::now();
      std::shared_ptr<U::CCLambda> lam(new U::CCLambda(cc, hbar));
      lam->compute_lambda();
      out.num("lambda_s", secs(ta, clk::now()));
      out.num("pseudoenergy", lam->pseudoenergy());
      out.mat("l1", lam->l1_, no, nv);
      out.t4("l2", lam->l2_, no, no, nv, nv);

      ta = clk::now();
      std::shared_ptr<U::CCDensity> dens(new U::CCDensity(cc, lam));
      const double eone = dens->onepdm();
      const double etwo = dens->twopdm();
      out.num("density_s", secs(ta, clk::now()));
      out.num("e_onepdm", eone);
      out.num("e_twopdm", etwo);
      out.mat("Doo", dens->Doo_, no, no);
      out.mat("Dvv", dens->Dvv_, nv, nv);
      out.mat("Dov", dens->Dov_, no, nv);
      out.mat("Dvo", dens->Dvo_, nv, no);
      // the six two-particle density blocks (ccdensity.cc:153-339)
      out.t4("Goooo", dens->Goooo_, no, no, no, no);
      out.t4("Gvvvv", dens->Gvvvv_, nv, nv, nv, nv);
      out.t4("Gooov", dens->Gooov_, no, no, no, nv);
      out.t4("Gvvvo", dens->Gvvvo_, nv, nv, nv, no);
      out.t4("Govov", dens->Govov_, no, nv, no, nv);
      out.t4("Goovv", dens->Goovv_, no, no, nv, nv);

      if (kv["DERTYPE"] == "SECOND") {
        if (in.npert < 6) throw std::runtime_error("response needs 3 dipole + 3 angular momentum matrices");
        // double** views of the perturbation matrices (3 Mu, then 3 L)
        std::vector<std::vector<double*> > rows(in.npert, std::vector<double*>(nact));
        std::vector<std::vector<double> > store = in.perts;
        for (int k = 0; k < in.npert; k++)
          for (int p = 0; p < nact; p++) rows[k][p] = store[k].data() + (size_t)p * nact;
        const double omega = options.get_double("MY_OMEGA");
        const bool lefthand = options.get_str("MYHAND") != "RIGHT";
        const char* cart = "XYZ";
        std::map<std::string, std::shared_ptr<U::CCPert> > perts;
        ta = clk::now();
        for (int x = 0; x < 3; x++) {
          std::string mu = std::string("Mu") + cart[x], am = std::string("L") + cart[x];
          perts[mu] = std::make_shared<U::CCPert>(rows[x].data(), omega, cc, hbar, lam);
          perts[mu]->solve(U::right);
          perts[am] = std::make_shared<U::CCPert>(rows[3 + x].data(), omega, cc, hbar, lam);
          perts[am]->solve(U::right);
          if (omega != 0.0 && !lefthand) {
            perts[mu + "-"] = std::make_shared<U::CCPert>(rows[x].data(), -omega, cc, hbar, lam);
            perts[mu + "-"]->solve(U::right);
          }
          if (lefthand) {
            // ugacc.cc:187-193 solves the left-hand equations for the most recent
            // entries; with omega != 0 in LEFT mode that is the +omega Mu solve.
            perts[mu]->solve(U::left);
            perts[am]->solve(U::left);
          }
        }
        out.num("response_solve_s", secs(ta, clk::now()));
        for (auto& kvp : perts) {
          out.mat("X1_" + kvp.first, kvp.second->X1_, no, nv);
          out.t4("X2_" + kvp.first, kvp.second->X2_, no, no, nv, nv);
          out.mat("Y1_" + kvp.first, kvp.second->Y1_, no, nv);
          out.t4("Y2_" + kvp.first, kvp.second->Y2_, no, no, nv, nv);
        }
        for (int p = 0; p < 3; p++)
          for (int q = 0; q <= p; q++) {
            auto P = perts[std::string("Mu") + cart[p]], Q = perts[std::string("Mu") + cart[q]];
            U::CCResp resp(P, Q);
            double polar;
            if (p == q)
              polar = resp.linresp(P, Q);
            else
              polar = 0.5 * resp.linresp(P, Q) + 0.5 * resp.linresp(Q, P);
            out.num(std::string("alpha_") + cart[p] + cart[q], polar);
          }
        for (int p = 0; p < 3; p++)
          for (int q = 0; q < 3; q++) {
            auto P = perts[std::string("Mu") + cart[p]], Q = perts[std::string("L") + cart[q]];
            U::CCResp resp(P, Q);
            double rot = 0.5 * resp.linresp(P, Q) - 0.5 * resp.linresp(Q, P);
            out.num(std::string("rot_") + cart[p] + cart[q], -rot);
          }
      }
    }
    out.num("total_s", secs(t0, clk::now()));
    out.str("status", "ok");
  } catch (const std::exception& e) {
    out.str("status", std::string("error: ") + e.what());
    out.finish();
    std::fprintf(stderr, "ugacc_ref: %s\n", e.what());
    return 1;
  }
  out.finish();
  std::fclose(logf);
  return 0;
}
