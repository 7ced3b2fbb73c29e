// C ABI (include/ugacc_gb300.h): argument checks, the exception boundary, stage order.
#include <cmath>
#include <cstring>

#include "cc.h"
#include "pert.h"

namespace ucc {
bool sliced_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                     const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi, int S);
void tc_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi);
void tc_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi, int parts,
                 int kc);
void wait_selftest(Ctx& c, unsigned long long limit_ns);
}

using namespace ucc;

struct ucc_ctx {
  Ctx c;
};

namespace ucc {
Ctx& ctx_of(ucc_ctx* h) { return h->c; }

Ctx::~Ctx() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto& t : gemm_timers) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  for (auto e : event_pool) cudaEventDestroy(e);
  anchors.clear();  // pool buffers are freed on the stream
  tc_cache.reset();
  perts.clear();
  store.clear();
  if (stream) cudaStreamDestroy(stream);
}
}  // namespace ucc

namespace {
template <typename F>
ucc_status guard(ucc_ctx* ctx, F&& f) {
  if (!ctx) return UCC_BAD_ARGS;
  ctx->c.last_error.clear();
  try {
    f(ctx->c);
    tc_check(ctx->c);  // deferred status of the tensor-core launches of this call
    return UCC_OK;
  } catch (const Error& e) {
    ctx->c.last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc& e) {
    ctx->c.last_error = "host allocation failed";
    return UCC_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    ctx->c.last_error = e.what();
    return UCC_CUDA_ERROR;
  }
}

void reset_state(Ctx& c) {
  cudaStreamSynchronize(c.stream);
  c.tc_cache.reset();
  c.perts.clear();
  c.store.clear();
  c.shapes.clear();
  c.loaded = c.have_ccsd = c.have_hbar = c.have_lambda = c.have_tgrad = false;
  // the old blocks went back to the stream-ordered pool, which keeps what it is given; hand
  // it to the device so that the cached tensor-core operands of the next Hamiltonian
  // (cudaMalloc) find it free (a second no=32/nv=320 load on one context otherwise spent
  // 4.4 s in its first record sweep)
  cudaMemPool_t pool;
  if (cudaStreamSynchronize(c.stream) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, c.device) == cudaSuccess)
    cudaMemPoolTrimTo(pool, 0);
}
}  // namespace

extern "C" {

void ucc_options_default(ucc_options* o) {
  if (!o) return;
  o->maxiter = 100;
  o->r_convergence = 1e-7;
  o->diis = 1;
  o->precision = UCC_FP64;
  o->refine_sweeps = 2;
  o->print = 0;
  o->mixed_switch = 1e-5;
  o->ooc = 0;
}

const char* ucc_status_string(ucc_status s) {
  switch (s) {
    case UCC_OK: return "ok";
    case UCC_NOT_CONVERGED: return "Computation has not converged.";
    case UCC_NAN_DETECTED: return "non-finite value detected";
    case UCC_OUT_OF_MEMORY: return "out of memory";
    case UCC_BAD_ARGS: return "bad arguments";
    case UCC_BAD_STATE: return "stage called before the stage it depends on";
    case UCC_CUDA_ERROR: return "CUDA error";
    case UCC_DEVICE_TIMEOUT: return "device-side wait timed out";
    case UCC_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

const char* ucc_last_error(ucc_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

ucc_status ucc_ctx_create(ucc_ctx** out, int device) {
  if (!out) return UCC_BAD_ARGS;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return UCC_CUDA_ERROR;
  ucc_ctx* ctx = new (std::nothrow) ucc_ctx;
  if (!ctx) return UCC_OUT_OF_MEMORY;
  ucc_status st = guard(ctx, [&](Ctx& c) {
    c.device = device;
    UCC_CUDA(cudaSetDevice(device));
    UCC_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    cudaMemPool_t pool;
    UCC_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;  // keep scratch cached between calls
    UCC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    ucc_options_default(&c.opt);
  });
  if (st != UCC_OK) {
    delete ctx;
    return st;
  }
  *out = ctx;
  return UCC_OK;
}

ucc_status ucc_ctx_destroy(ucc_ctx* ctx) {
  if (!ctx) return UCC_BAD_ARGS;
  const int device = ctx->c.device;
  cudaSetDevice(device);
  cudaStreamSynchronize(ctx->c.stream);
  delete ctx;
  // the context's scratch went back to the device's stream-ordered pool, which keeps it
  // (release threshold: keep); hand it back to the device so that later cudaMalloc calls
  // (cached tensor-core operands of the next context) can use it
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    cudaDeviceSynchronize();
    cudaMemPoolTrimTo(pool, 0);
  }
  return UCC_OK;
}

ucc_status ucc_set_options(ucc_ctx* ctx, const ucc_options* o) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(o, UCC_BAD_ARGS, "null options");
    UCC_REQUIRE(o->maxiter >= 1, UCC_BAD_ARGS, "maxiter must be >= 1");
    UCC_REQUIRE(o->r_convergence > 0, UCC_BAD_ARGS, "r_convergence must be > 0");
    UCC_REQUIRE(o->precision == UCC_FP64 || o->precision == UCC_MIXED, UCC_BAD_ARGS, "bad precision");
    UCC_REQUIRE(o->refine_sweeps >= 0, UCC_BAD_ARGS, "refine_sweeps must be >= 0");
    UCC_REQUIRE(o->mixed_switch > 0, UCC_BAD_ARGS, "mixed_switch must be > 0");
    UCC_REQUIRE(o->ooc == 0 || o->ooc == 1, UCC_BAD_ARGS, "ooc must be 0 or 1");
    c.opt = *o;
  });
}

ucc_status ucc_load_hamiltonian(ucc_ctx* ctx, int no, int nv, const double* fock, const double* ints) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(no >= 1 && nv >= 1 && fock && ints, UCC_BAD_ARGS, "need no >= 1, nv >= 1, fock and ints");
    UCC_CUDA(cudaSetDevice(c.device));
    reset_state(c);
    load_from_ints(c, no, nv, fock, ints);
    c.loaded = true;
  });
}

ucc_status ucc_load_hamiltonian_df(ucc_ctx* ctx, int no, int nv, int naux, const double* fock, const double* B) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(no >= 1 && nv >= 1 && naux >= 1 && fock && B, UCC_BAD_ARGS, "need no, nv, naux >= 1, fock and B");
    UCC_CUDA(cudaSetDevice(c.device));
    reset_state(c);
    load_from_df(c, no, nv, naux, fock, B);
    c.loaded = true;
  });
}

ucc_status ucc_ccsd(ucc_ctx* ctx, double* e, int* iters) {
  bool conv = true;
  ucc_status st = guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    CCSDResult r = run_ccsd(c);
    c.stats.ccsd_ms += tm.stop_ms();
    c.stats.ccsd_iterations = r.iterations;
    c.stats.ccsd_flops += flops_ccsd_iter(c.no, c.nv) * r.iterations;
    c.stats.kernel_launches += launches() - l0;
    if (e) *e = r.e_ccsd;
    if (iters) *iters = r.iterations;
    conv = r.converged;
  });
  if (st == UCC_OK && !conv) {
    ctx->c.last_error = "Computation has not converged.";
    return UCC_NOT_CONVERGED;
  }
  return st;
}

ucc_status ucc_triples(ucc_ctx* ctx, double* et) {
  return guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    const double e = run_triples(c);
    c.stats.triples_ms += tm.stop_ms();
    c.stats.triples_flops += flops_triples(c.no, c.nv);
    c.stats.kernel_launches += launches() - l0;
    if (et) *et = e;
  });
}

ucc_status ucc_triples_gradient(ucc_ctx* ctx) {
  return guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    run_triples_gradient(c);
    c.stats.triples_ms += tm.stop_ms();
    c.stats.kernel_launches += launches() - l0;
  });
}

ucc_status ucc_hbar(ucc_ctx* ctx) {
  return guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    run_hbar(c);
    c.stats.hbar_ms += tm.stop_ms();
    c.stats.kernel_launches += launches() - l0;
  });
}

ucc_status ucc_lambda(ucc_ctx* ctx, double* pseudo, int* iters) {
  bool conv = true;
  ucc_status st = guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    CCSDResult r = run_lambda(c);
    c.stats.lambda_ms += tm.stop_ms();
    c.stats.lambda_iterations = r.iterations;
    c.stats.kernel_launches += launches() - l0;
    if (pseudo) *pseudo = r.e_ccsd;
    if (iters) *iters = r.iterations;
    conv = r.converged;
  });
  if (st == UCC_OK && !conv) {
    ctx->c.last_error = "Computation has not converged.";
    return UCC_NOT_CONVERGED;
  }
  return st;
}

ucc_status ucc_density(ucc_ctx* ctx, double* e1, double* e2) {
  return guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    double a = 0, b = 0;
    run_density(c, &a, &b);
    c.stats.density_ms += tm.stop_ms();
    c.stats.kernel_launches += launches() - l0;
    if (e1) *e1 = a;
    if (e2) *e2 = b;
  });
}

ucc_status ucc_twopdm_energies(ucc_ctx* ctx, double* parts) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(parts, UCC_BAD_ARGS, "null output");
    UCC_REQUIRE(c.has("Goooo"), UCC_BAD_STATE, "no densities computed (ucc_density first)");
    for (int k = 0; k < 6; k++) parts[k] = c.e2_parts[k];
  });
}

ucc_status ucc_pert_create(ucc_ctx* ctx, const double* pert, double omega, int* handle) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(pert && handle && std::isfinite(omega), UCC_BAD_ARGS, "need pert, handle and a finite omega");
    UCC_CUDA(cudaSetDevice(c.device));
    *handle = pert_create(c, pert, omega);
  });
}

ucc_status ucc_pert_solve(ucc_ctx* ctx, int handle, int hand, double* pseudo, int* iters) {
  bool conv = true;
  ucc_status st = guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(hand == 0 || hand == 1, UCC_BAD_ARGS, "hand must be 0 (left) or 1 (right)");
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    Timer tm(c.stream);
    tm.start();
    CCSDResult r = pert_solve(c, handle, hand == 1);
    c.stats.pert_ms += tm.stop_ms();
    c.stats.kernel_launches += launches() - l0;
    if (pseudo) *pseudo = r.e_ccsd;
    if (iters) *iters = r.iterations;
    conv = r.converged;
  });
  if (st == UCC_OK && !conv) {
    ctx->c.last_error = "Computation has not converged.";
    return UCC_NOT_CONVERGED;
  }
  return st;
}

ucc_status ucc_linresp(ucc_ctx* ctx, int hx, int hy, double* value) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(value, UCC_BAD_ARGS, "null output");
    UCC_CUDA(cudaSetDevice(c.device));
    const int64_t l0 = launches();
    *value = linresp(c, hx, hy);
    c.stats.kernel_launches += launches() - l0;
  });
}

static ucc_status gemm_host(ucc_ctx* ctx, int precision, int digits, int transa, int transb, int64_t M, int64_t N,
                            int64_t K, double alpha, const double* A, const double* B, double beta, double* C) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(A && B && C && M >= 1 && N >= 1 && K >= 1, UCC_BAD_ARGS, "ucc_gemm: bad arguments");
    UCC_REQUIRE(digits >= 2 && digits <= 9, UCC_BAD_ARGS, "ucc_gemm_sliced: 2 to 9 digits");
    UCC_REQUIRE(precision == UCC_FP64 || precision == UCC_MIXED || precision == UCC_MIXED_FINE ||
                    precision == UCC_FP64_SLICED,
                UCC_BAD_ARGS, "ucc_gemm: bad precision");
    UCC_CUDA(cudaSetDevice(c.device));
    Scratch dA(c, sizeof(double) * M * K), dB(c, sizeof(double) * K * N), dC(c, sizeof(double) * M * N);
    UCC_CUDA(cudaMemcpyAsync(dA.p, A, sizeof(double) * M * K, cudaMemcpyHostToDevice, c.stream));
    UCC_CUDA(cudaMemcpyAsync(dB.p, B, sizeof(double) * K * N, cudaMemcpyHostToDevice, c.stream));
    UCC_CUDA(cudaMemcpyAsync(dC.p, C, sizeof(double) * M * N, cudaMemcpyHostToDevice, c.stream));
    const int64_t sAm = transa ? 1 : K, sAk = transa ? M : 1;
    const int64_t sBk = transb ? 1 : N, sBn = transb ? K : 1;
    GemmEpilogue epi;
    epi.s_mhi = N;
    epi.s_n = 1;
    if (precision == UCC_MIXED)
      tc_gemm_run(c, M, N, K, alpha, dA.d(), sAm, sAk, dB.d(), sBk, sBn, beta, dC.d(), epi);
    else if (precision == UCC_MIXED_FINE)
      tc_gemm_run(c, M, N, K, alpha, dA.d(), sAm, sAk, dB.d(), sBk, sBn, beta, dC.d(), epi, 3, 16);
    else if (precision == UCC_FP64_SLICED)
      UCC_REQUIRE(sliced_gemm_run(c, M, N, K, alpha, dA.d(), sAm, sAk, dB.d(), sBk, sBn, beta, dC.d(), epi, digits),
                  UCC_BAD_ARGS, "ucc_gemm: operands outside the sliced form's range (row maxima >= 2^498 or |alpha| "
                                "outside [2^-20, 2^20])");
    else
      dgemm_strided(c, M, N, K, alpha, dA.d(), sAm, sAk, dB.d(), sBk, sBn, beta, dC.d(), epi, 1, 0, 0, 0, nullptr);
    UCC_CUDA(cudaMemcpyAsync(C, dC.p, sizeof(double) * M * N, cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
  });
}

ucc_status ucc_gemm(ucc_ctx* ctx, int precision, int transa, int transb, int64_t M, int64_t N, int64_t K,
                    double alpha, const double* A, const double* B, double beta, double* C) {
  return gemm_host(ctx, precision, 9, transa, transb, M, N, K, alpha, A, B, beta, C);
}

ucc_status ucc_gemm_sliced(ucc_ctx* ctx, int digits, int transa, int transb, int64_t M, int64_t N, int64_t K,
                           double alpha, const double* A, const double* B, double beta, double* C) {
  return gemm_host(ctx, UCC_FP64_SLICED, digits, transa, transb, M, N, K, alpha, A, B, beta, C);
}

ucc_status ucc_wait_selftest(ucc_ctx* ctx, uint64_t limit_ns) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(limit_ns >= 1000 && limit_ns <= 10000000000ull, UCC_BAD_ARGS,
                "ucc_wait_selftest: limit between 1 us and 10 s");
    UCC_CUDA(cudaSetDevice(c.device));
    wait_selftest(c, (unsigned long long)limit_ns);
  });
}

ucc_status ucc_get_tensor(ucc_ctx* ctx, const char* name, double* out, size_t count) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(name && out, UCC_BAD_ARGS, "null argument");
    UCC_CUDA(cudaSetDevice(c.device));
    Tensor t = named_tensor(c, name);
    UCC_REQUIRE((size_t)t.size() == count, UCC_BAD_ARGS,
                std::string("size mismatch for ") + name + ": expected " + std::to_string(t.size()));
    Tensor tmp = t;
    std::unique_ptr<Scratch> hold;
    if (!t.dense()) {
      std::vector<int64_t> dims(t.d, t.d + t.rank);
      hold = std::make_unique<Scratch>(c, sizeof(double) * t.size());
      tmp = make_view(hold->d(), dims);
      permute_add(c, t, 1.0, 0.0, tmp);
    }
    UCC_CUDA(cudaMemcpyAsync(out, tmp.p, sizeof(double) * count, cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
  });
}

ucc_status ucc_set_tensor(ucc_ctx* ctx, const char* name, const double* in, size_t count) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(name && in, UCC_BAD_ARGS, "null argument");
    UCC_REQUIRE(c.loaded, UCC_BAD_STATE, "no Hamiltonian loaded");
    UCC_CUDA(cudaSetDevice(c.device));
    set_named_tensor(c, name, in, count);
  });
}

ucc_status ucc_get_stats(ucc_ctx* ctx, ucc_stats* out) {
  return guard(ctx, [&](Ctx& c) {
    UCC_REQUIRE(out, UCC_BAD_ARGS, "null output");
    UCC_CUDA(cudaSetDevice(c.device));
    c.resolve_timers();
    *out = c.stats;
  });
}

ucc_status ucc_reset_stats(ucc_ctx* ctx) {
  return guard(ctx, [&](Ctx& c) {
    UCC_CUDA(cudaSetDevice(c.device));
    c.resolve_timers();
    c.stats = ucc_stats{};
  });
}

}  // extern "C"
