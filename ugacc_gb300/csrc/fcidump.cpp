// Hamiltonian from an MO-integral file (host code, no device work).
//
// The reference builds its Hamiltonian from psi4 (hamiltonian.cc:21-102): the Fock matrix
// of the reference determinant over the active orbitals in QT order (occupied first,
// :43-56), the two-electron integrals <pq|rs> = (pr|qs) over the active orbitals
// (:76-91, ints_[p][r][q][s] = (pq|rs)) and the frozen-core energy (:72), with frozen
// core and frozen virtual orbitals removed (:24-27).  This file does the same from a text
// file in the FCIDUMP layout, for hosts that have MO integrals but no psi4:
//
//   header   &FCI NORB=n, NELEC=N, MS2=0, [ORBSYM=...,] [ISYM=...,] [UHF=.FALSE.,] &END
//            (or a line "/" as the terminator)
//   body     value i j k l    i,j,k,l >= 1: (ij|kl), real orbitals, any one of the 8
//                             equivalent index orders
//            value i j 0 0    h_ij (one-electron operator, symmetric)
//            value i 0 0 0    orbital energy
//            value 0 0 0 0    nuclear repulsion energy
//   values may use a Fortran D exponent (1.0D-02).
//
// Orbital order: when every orbital has an energy line, the NELEC/2 lowest are doubly
// occupied and the orbitals are put in QT order, occupied then virtual, each by ascending
// energy (a stable sort: an energy-ordered file keeps its order; files grouped by irrep,
// as symmetry-using programs write them, are regrouped).  Otherwise the file's order is
// taken with the first NELEC/2 occupied.  The first nfzc orbitals of that order are
// frozen core and the last nfzv frozen virtuals.  The reference's reorder_qt (frozen
// docc, docc, virtuals, frozen virtuals, hamiltonian.cc:40-41) also orders each class by
// irrep; the CC energies do not depend on the order within the occupied or the virtual
// space.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <algorithm>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ugacc_gb300.h"

namespace {

struct DumpError : std::runtime_error {
  ucc_status status;
  DumpError(ucc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

struct Header {
  int norb = -1, nelec = -1, ms2 = 0;
  bool uhf = false;
  size_t body = 0;  // offset of the first byte after the header
};

std::string read_file(const char* path) {
  if (!path) throw DumpError(UCC_BAD_ARGS, "fcidump: null path");
  std::ifstream f(path, std::ios::binary);
  if (!f) throw DumpError(UCC_BAD_ARGS, std::string("fcidump: cannot open ") + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

std::string upper(std::string s) {
  for (auto& ch : s) ch = (char)std::toupper((unsigned char)ch);
  return s;
}

// value of KEY= in the header text (upper case), or "" when absent
std::string key_value(const std::string& hdr, const char* key) {
  const std::string k = std::string(key) + "=";
  size_t p = 0;
  while ((p = hdr.find(k, p)) != std::string::npos) {
    // a whole key: not the tail of a longer name (e.g. ISYM inside ORBSYM)
    if (p == 0 || !std::isalnum((unsigned char)hdr[p - 1])) break;
    p += k.size();
  }
  if (p == std::string::npos) return "";
  p += k.size();
  while (p < hdr.size() && std::isspace((unsigned char)hdr[p])) p++;
  size_t q = p;
  while (q < hdr.size() && hdr[q] != ',' && !std::isspace((unsigned char)hdr[q]) && hdr[q] != '&' && hdr[q] != '/')
    q++;
  return hdr.substr(p, q - p);
}

Header parse_header(const std::string& text) {
  Header h;
  const std::string up = upper(text.substr(0, std::min<size_t>(text.size(), 1 << 20)));
  if (up.find("&FCI") == std::string::npos) throw DumpError(UCC_BAD_ARGS, "fcidump: no &FCI header");
  // the header ends at &END (or /END) or at a line holding only "/"
  size_t end = std::string::npos, after = 0;
  const size_t e1 = up.find("&END"), e2 = up.find("/END");
  if (e1 != std::string::npos || e2 != std::string::npos) {
    end = std::min(e1, e2);
    after = end + 4;
  } else {
    size_t p = 0;
    while (p < up.size()) {
      size_t nl = up.find('\n', p);
      if (nl == std::string::npos) nl = up.size();
      std::string line = up.substr(p, nl - p);
      const size_t a = line.find_first_not_of(" \t\r"), b = line.find_last_not_of(" \t\r");
      if (a != std::string::npos && line.substr(a, b - a + 1) == "/") {
        end = p;
        after = nl;
        break;
      }
      p = nl + 1;
    }
  }
  if (end == std::string::npos) throw DumpError(UCC_BAD_ARGS, "fcidump: header has no &END or / terminator");
  const std::string hdr = up.substr(0, end);
  const std::string norb = key_value(hdr, "NORB"), nelec = key_value(hdr, "NELEC");
  if (norb.empty() || nelec.empty()) throw DumpError(UCC_BAD_ARGS, "fcidump: NORB and NELEC are required");
  h.norb = std::atoi(norb.c_str());
  h.nelec = std::atoi(nelec.c_str());
  const std::string ms2 = key_value(hdr, "MS2");
  if (!ms2.empty()) h.ms2 = std::atoi(ms2.c_str());
  const std::string uhf = key_value(hdr, "UHF");
  h.uhf = !uhf.empty() && (uhf.find('T') != std::string::npos || uhf == "1");
  if (h.norb <= 0 || h.nelec < 0) throw DumpError(UCC_BAD_ARGS, "fcidump: bad NORB or NELEC");
  h.body = after;
  return h;
}

// next number of the body (Fortran D exponents accepted); false at the end
bool next_number(const char*& p, const char* end, double& v, std::string& tmp) {
  while (p < end && (std::isspace((unsigned char)*p) || *p == ',')) p++;
  if (p >= end) return false;
  const char* q = p;
  while (q < end && !std::isspace((unsigned char)*q) && *q != ',') q++;
  tmp.assign(p, q);
  for (auto& ch : tmp)
    if (ch == 'D' || ch == 'd') ch = 'E';
  char* stop = nullptr;
  v = std::strtod(tmp.c_str(), &stop);
  if (stop == tmp.c_str() || *stop != '\0') throw DumpError(UCC_BAD_ARGS, "fcidump: bad number '" + tmp + "'");
  p = q;
  return true;
}

struct Integrals {
  int n = 0;
  std::vector<double> h, eri;  // h[n][n]; eri[n][n][n][n] = (pq|rs)
  std::vector<double> eorb;    // orbital energies, when given
  std::vector<char> has_e;
  double enuc = 0.0;
  double& g(int p, int q, int r, int s) { return eri[(((size_t)p * n + q) * n + r) * n + s]; }
};

void read_body(const std::string& text, size_t off, Integrals& I) {
  const int n = I.n;
  I.h.assign((size_t)n * n, 0.0);
  I.eri.assign((size_t)n * n * n * n, 0.0);
  I.eorb.assign(n, 0.0);
  I.has_e.assign(n, 0);
  const char* p = text.data() + off;
  const char* end = text.data() + text.size();
  std::string tmp;
  double f[5];
  for (;;) {
    if (!next_number(p, end, f[0], tmp)) break;
    for (int k = 1; k < 5; k++)
      if (!next_number(p, end, f[k], tmp)) throw DumpError(UCC_BAD_ARGS, "fcidump: truncated integral line");
    int x[4];
    for (int k = 0; k < 4; k++) {
      if (!(f[k + 1] >= 0.0 && f[k + 1] <= (double)n) || std::floor(f[k + 1]) != f[k + 1])
        throw DumpError(UCC_BAD_ARGS, "fcidump: orbital index out of range");
      x[k] = (int)f[k + 1];
    }
    const double v = f[0];
    const int i = x[0] - 1, j = x[1] - 1, k = x[2] - 1, l = x[3] - 1;
    if (x[0] && x[1] && x[2] && x[3]) {
      I.g(i, j, k, l) = v, I.g(j, i, k, l) = v, I.g(i, j, l, k) = v, I.g(j, i, l, k) = v;
      I.g(k, l, i, j) = v, I.g(l, k, i, j) = v, I.g(k, l, j, i) = v, I.g(l, k, j, i) = v;
    } else if (x[0] && x[1] && !x[2] && !x[3]) {
      I.h[(size_t)i * n + j] = v;
      I.h[(size_t)j * n + i] = v;
    } else if (!x[0] && !x[1] && !x[2] && !x[3]) {
      I.enuc = v;
    } else if (x[0] && !x[1] && !x[2] && !x[3]) {
      I.eorb[i] = v;
      I.has_e[i] = 1;
    } else {
      throw DumpError(UCC_BAD_ARGS, "fcidump: unrecognised index pattern");
    }
  }
}

void set_error(char* err, size_t errlen, const char* msg) {
  if (err && errlen) {
    std::strncpy(err, msg, errlen - 1);
    err[errlen - 1] = '\0';
  }
}

template <typename F>
ucc_status dump_guard(char* err, size_t errlen, F&& f) {
  set_error(err, errlen, "");
  try {
    f();
    return UCC_OK;
  } catch (const DumpError& e) {
    set_error(err, errlen, e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_error(err, errlen, "fcidump: host allocation failed (the file's NORB^4 integral array)");
    return UCC_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_error(err, errlen, e.what());
    return UCC_BAD_ARGS;
  }
}

}  // namespace

extern "C" {

ucc_status ucc_fcidump_dims(const char* path, int* norb, int* nelec, char* err, size_t errlen) {
  return dump_guard(err, errlen, [&] {
    if (!norb || !nelec) throw DumpError(UCC_BAD_ARGS, "fcidump: null output");
    const Header h = parse_header(read_file(path));
    *norb = h.norb;
    *nelec = h.nelec;
  });
}

ucc_status ucc_fcidump_read(const char* path, int nfzc, int nfzv, double* fock, double* ints, double* energies,
                            int* order, char* err, size_t errlen) {
  return dump_guard(err, errlen, [&] {
    if (!fock || !ints || !energies) throw DumpError(UCC_BAD_ARGS, "fcidump: null output");
    const std::string text = read_file(path);
    const Header hd = parse_header(text);
    if (hd.uhf || hd.ms2 != 0 || hd.nelec % 2 != 0)
      throw DumpError(UCC_UNSUPPORTED, "fcidump: closed-shell RHF integrals only (MS2=0, even NELEC, no UHF)");
    const int n = hd.norb, nocc = hd.nelec / 2;
    if (nocc > n) throw DumpError(UCC_BAD_ARGS, "fcidump: NELEC/2 exceeds NORB");
    if (nfzc < 0 || nfzv < 0 || nfzc >= nocc || nfzv >= n - nocc)
      throw DumpError(UCC_BAD_ARGS, "fcidump: frozen orbitals leave no active occupied or virtual orbital");
    Integrals I;
    I.n = n;
    read_body(text, hd.body, I);
    // qt[P] = the file's orbital at QT position P
    std::vector<int> qt(n);
    std::iota(qt.begin(), qt.end(), 0);
    if (std::all_of(I.has_e.begin(), I.has_e.end(), [](char c) { return c != 0; })) {
      std::stable_sort(qt.begin(), qt.end(), [&](int a, int b) { return I.eorb[a] < I.eorb[b]; });
      // (ascending energy: the NELEC/2 lowest come first, each class stays in energy order)
    }
    auto h = [&](int p, int q) { return I.h[(size_t)qt[p] * n + qt[q]]; };
    auto g = [&](int p, int q, int r, int s) { return I.g(qt[p], qt[q], qt[r], qt[s]); };
    // Fock matrix of the determinant with QT orbitals 0..nocc-1 doubly occupied (frozen
    // core included): F_pq = h_pq + sum_k [2 (pq|kk) - (pk|kq)]
    std::vector<double> F((size_t)n * n);
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) {
        double s = h(p, q);
        for (int k = 0; k < nocc; k++) s += 2.0 * g(p, q, k, k) - g(p, k, k, q);
        F[(size_t)p * n + q] = s;
      }
    // frozen-core energy: sum_i [2 h_ii + sum_j (2 (ii|jj) - (ij|ji))] over frozen i, j
    double efzc = 0.0;
    for (int i = 0; i < nfzc; i++) {
      efzc += 2.0 * h(i, i);
      for (int j = 0; j < nfzc; j++) efzc += 2.0 * g(i, i, j, j) - g(i, j, j, i);
    }
    double escf = I.enuc;
    for (int k = 0; k < nocc; k++) escf += h(k, k) + F[(size_t)k * n + k];
    const int a0 = nfzc, na = n - nfzc - nfzv;
    for (int p = 0; p < na; p++)
      for (int q = 0; q < na; q++) fock[(size_t)p * na + q] = F[(size_t)(a0 + p) * n + a0 + q];
    // <pq|rs> = (pr|qs): the reference's ints_[p][r][q][s] = (pq|rs)
    for (int p = 0; p < na; p++)
      for (int q = 0; q < na; q++)
        for (int r = 0; r < na; r++)
          for (int s = 0; s < na; s++)
            ints[(((size_t)p * na + q) * na + r) * na + s] = g(a0 + p, a0 + r, a0 + q, a0 + s);
    if (order)  // the file's (0-based) orbital at each active QT position
      for (int p = 0; p < na; p++) order[p] = qt[a0 + p];
    energies[0] = I.enuc;
    energies[1] = efzc;
    energies[2] = escf;
  });
}

}  // extern "C"
