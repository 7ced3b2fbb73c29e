/*
 * C ABI of the GB300 (sm_103a) RHF coupled-cluster library.
 *
 * The reference is a psi4 plugin whose hot path is a stack of C++ classes
 * (ugacc hamiltonian.h:12-34, ccwfn.h:12-106, hbar.h:11-36, cclambda.h:13-63,
 * ccdensity.h:12-50, ccpert.h:17-80, ccresp.h:10-28) that share raw double**** arrays.
 * This header is the boundary those classes are rebuilt on: plain pointers and sizes,
 * no C++ or torch types, every call returns a ucc_status and never throws.
 *
 * Array layouts (row-major, float64, host memory unless stated):
 *   fock        [nact][nact], occupied orbitals first (QT order), nact = no + nv
 *   ints        [nact][nact][nact][nact], ints[p][q][r][s] = <pq|rs> = (pr|qs)
 *   B           [naux][nact][nact], (pq|rs) = sum_Q B[Q][p][q] B[Q][r][s]
 *   t1, l1, X1, Y1     [no][nv];    t2, l2, X2, Y2    [no][no][nv][nv]
 *   pert        [nact][nact] one-electron perturbation matrix
 */
#ifndef UGACC_GB300_H
#define UGACC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ucc_status {
  UCC_OK = 0,
  UCC_NOT_CONVERGED = 1,   /* reference: PSIEXCEPTION("Computation has not converged.") */
  UCC_NAN_DETECTED = 2,
  UCC_OUT_OF_MEMORY = 3,
  UCC_BAD_ARGS = 4,
  UCC_BAD_STATE = 5,       /* a stage was called before the stage it depends on */
  UCC_CUDA_ERROR = 6,
  UCC_DEVICE_TIMEOUT = 7,  /* a bounded device-side wait gave up */
  UCC_UNSUPPORTED = 8
} ucc_status;

typedef struct ucc_ctx ucc_ctx;

/* Arithmetic of the contractions. FP64 is the plain form; MIXED runs the large
 * contractions (particle ladder, rings, (T)) as BF16 hi+lo split products with FP32
 * accumulation on the tensor cores and keeps denominators, updates, DIIS, norms and
 * energies in FP64, followed by FP64 refinement sweeps. */
typedef enum ucc_precision {
  UCC_FP64 = 0,
  UCC_MIXED = 1,
  UCC_MIXED_FINE = 2, /* ucc_gemm only: three-part split, K in FP64-summed chunks (refinement corrections) */
  UCC_FP64_SLICED = 3 /* ucc_gemm only: FP64-accurate product of exact bf16 slices on the tensor cores (the
                         form the FP64 work of MIXED solves runs in) */
} ucc_precision;

/* Solver options: the reference's psi4 options (ugacc.cc:57-68) plus the new ones. */
typedef struct ucc_options {
  int maxiter;            /* MAXITER, default 100 */
  double r_convergence;   /* R_CONVERGENCE on the 2-norm of the residual, default 1e-7 */
  int diis;               /* DIIS on/off, default 1 (8 vectors) */
  int precision;          /* ucc_precision, default UCC_FP64 */
  int refine_sweeps;      /* FP64 sweeps after a MIXED solve, default 2 */
  int print;              /* 0 silent, 1 iteration table on stdout */
  double mixed_switch;    /* MIXED: residual norm at which FP64 sweeps take over, default 1e-5 */
  int ooc;                /* OOC, default 0 as the plugin (ugacc.cc:67): the (T) gradient's Doo and Dvv
                             are full matrices (tgrad, ccwfn.cc:998-1021); 1: their diagonals only
                             (tgrad_ooc, ccwfn.cc:1203,1247). Every other piece is the same. */
} ucc_options;

void ucc_options_default(ucc_options* opt);

/* Replaces: psi::ugacc::Hamiltonian::Hamiltonian (hamiltonian.cc:19-104). */
ucc_status ucc_ctx_create(ucc_ctx** ctx, int device);
ucc_status ucc_ctx_destroy(ucc_ctx* ctx);
ucc_status ucc_set_options(ucc_ctx* ctx, const ucc_options* opt);
ucc_status ucc_load_hamiltonian(ucc_ctx* ctx, int no, int nv, const double* fock, const double* ints);
ucc_status ucc_load_hamiltonian_df(ucc_ctx* ctx, int no, int nv, int naux, const double* fock, const double* B);

/* Replaces: the integral side of psi::ugacc::Hamiltonian::Hamiltonian (hamiltonian.cc:21-102)
 * for hosts with MO integrals in a file instead of psi4's libtrans.  The file has the
 * FCIDUMP layout: a header "&FCI NORB=n, NELEC=N, MS2=0, ... &END" (or a "/" line), then
 * lines "value i j k l" with (ij|kl) over real orbitals (1-based, any of the 8 equivalent
 * orders), "value i j 0 0" = h_ij, "value i 0 0 0" = orbital energy, "value 0 0 0 0" =
 * nuclear repulsion.  With an energy for every orbital, the NELEC/2 lowest are doubly
 * occupied and the orbitals go to QT order (occupied, then virtual, each by ascending
 * energy); otherwise the file's order is taken with the first NELEC/2 occupied.  The first
 * nfzc orbitals of that order are frozen core and the last nfzv frozen virtuals
 * (hamiltonian.cc:24-27).  Host code only: no context and no device needed.
 *   ucc_fcidump_dims: NORB and NELEC of the header.
 *   ucc_fcidump_read: fock [nact][nact] (the determinant's Fock matrix over the active
 *     orbitals, QT order, hamiltonian.cc:43-56), ints [nact]^4 with ints[p][q][r][s] =
 *     <pq|rs> = (pr|qs) (hamiltonian.cc:76-91), energies[3] = {nuclear repulsion,
 *     frozen-core energy (hamiltonian.cc:72), SCF energy}, order [nact] (may be null) the
 *     file's 0-based orbital at each active QT position, for cutting the same block out
 *     of the host's own MO-basis matrices (e.g. the perturbations of ucc_pert_create);
 *     nact = NORB - nfzc - nfzv, no = NELEC/2 - nfzc.  Closed-shell files only
 *     (UCC_UNSUPPORTED otherwise).
 * Errors are written to err (errlen bytes, may be null). */
ucc_status ucc_fcidump_dims(const char* path, int* norb, int* nelec, char* err, size_t errlen);
ucc_status ucc_fcidump_read(const char* path, int nfzc, int nfzv, double* fock, double* ints, double* energies,
                            int* order, char* err, size_t errlen);

/* Replaces: CCWfn::CCWfn + CCWfn::compute_energy, CCSD part (ccwfn.cc:12-120, :188-235).
 * e_ccsd is the energy of the amplitudes before the final update, as the reference
 * reports it (ccwfn.cc:224,233). */
ucc_status ucc_ccsd(ucc_ctx* ctx, double* e_ccsd, int* iterations);

/* Replaces: CCWfn::tcorr_ooc_TJL (ccwfn.cc:795-852) with W3_ijk (:1388-1418); the value
 * equals tcorr_ooc (:745-793) and tcorr (:647-743). */
ucc_status ucc_triples(ucc_ctx* ctx, double* e_t);

/* Replaces: CCWfn::tgrad (ccwfn.cc:854-1142, OOC=0) and CCWfn::tgrad_ooc (:1150-1316, OOC=1),
 * run by compute_energy for WFN=CCSD_T, DERTYPE=FIRST (:252-255): the (T) pieces of the
 * CCSD(T) first derivatives, computed triple by triple in both cases (T3/L3 are never stored).
 * Afterwards ucc_lambda adds s1 / s2/2 to its residuals (cclambda.cc:181,243) and
 * ucc_density starts from the (T) parts of Doo, Dvv, Dov, Goovv, Gooov, Gvvvo
 * (ccdensity.cc:44-69), until the next ucc_ccsd.  Tensors: "s1" "s2" "DooT" "DvvT" "DovT"
 * "GoovvT" "GooovT" "GvvvoT" (reference array layouts). */
ucc_status ucc_triples_gradient(ucc_ctx* ctx);

/* Replaces: HBAR::HBAR (hbar.cc:8-228). */
ucc_status ucc_hbar(ucc_ctx* ctx);

/* Replaces: CCLambda::CCLambda + compute_lambda (cclambda.cc:13-45, :93-129). */
ucc_status ucc_lambda(ucc_ctx* ctx, double* pseudoenergy, int* iterations);

/* Replaces: CCDensity::onepdm + twopdm (ccdensity.cc:89-339).  Afterwards the one- and
 * two-particle density blocks are tensors of the context: "Doo" "Dvv" "Dov" "Dvo" and
 * "Goooo" "Gooov" "Gvvvo" "Govov" "Goovv" (the (T) pieces included for WFN=CCSD_T with
 * DERTYPE=FIRST, as the reference starts them, ccdensity.cc:44-69), plus "Gvvvv" while
 * nv^4 <= 2^25 (its energy is formed without it). */
ucc_status ucc_density(ucc_ctx* ctx, double* e_onepdm, double* e_twopdm);
/* The six two-particle density energies the reference prints (ccdensity.cc:181-335), in
 * the order OOOO VVVV OOOV VVVO OVOV OOVV; their sum is ucc_density's e_twopdm. */
ucc_status ucc_twopdm_energies(ucc_ctx* ctx, double* parts6);

/* Replaces: CCPert::CCPert (ccpert.cc:11-77); returns a handle >= 0. */
ucc_status ucc_pert_create(ucc_ctx* ctx, const double* pert, double omega, int* handle);
/* Replaces: CCPert::solve (ccpert.cc:177-229); hand 0 = left, 1 = right (ccpert.h:15). */
ucc_status ucc_pert_solve(ucc_ctx* ctx, int handle, int hand, double* pseudoresponse, int* iterations);
/* Replaces: CCResp::linresp(X, Y) (ccresp.cc:28-124). */
ucc_status ucc_linresp(ucc_ctx* ctx, int handle_x, int handle_y, double* value);

/* C = alpha * op(A) op(B) + beta * C on host row-major float64 buffers, computed by the
 * library's FP64 GEMM (precision UCC_FP64) or its tensor-core BF16 hi+lo split GEMM
 * (UCC_MIXED, FP32 accumulation).  No counterpart in the reference (its contractions are
 * inline loops); this is the building block every contraction above runs on.
 * op(A) is M x K (transa: A stored K x M), op(B) is K x N (transb: B stored N x K). */
ucc_status ucc_gemm(ucc_ctx* ctx, int precision, int transa, int transb, int64_t M, int64_t N, int64_t K,
                    double alpha, const double* A, const double* B, double beta, double* C);

/* ucc_gemm with precision UCC_FP64_SLICED and `digits` (2 to 9) base-2^6 digits per operand
 * in place of 9: each operand row is truncated to 6*digits bits relative to its largest
 * element, so the error per product term is near 2^(-6*digits) of max|A row| * max|B col|.
 * The mixed-precision solvers use fewer digits for FP64 anchors whose delta sweeps only need
 * to resolve a residual well above r_convergence; the sweep that ends a solve uses 9. */
ucc_status ucc_gemm_sliced(ucc_ctx* ctx, int digits, int transa, int transb, int64_t M, int64_t N, int64_t K,
                           double alpha, const double* A, const double* B, double beta, double* C);

/* Failure-detection self-test (no counterpart in the reference, which has no device
 * code).  Every wait inside the tensor-core pipelines is bounded: when one runs out the
 * kernel raises a device flag and returns, and the call reports UCC_DEVICE_TIMEOUT.  This
 * entry point runs that path on purpose: one thread waits limit_ns (1 us to 10 s) on a
 * barrier that nothing completes.  Expected result: UCC_DEVICE_TIMEOUT, with the context
 * and its stream still usable for the next call. */
ucc_status ucc_wait_selftest(ucc_ctx* ctx, uint64_t limit_ns);

/* (T) correction computed without allocating any device memory.  No counterpart in the
 * reference: it serves host programs that cannot let a library call cudaMalloc (all
 * device memory belongs to their own arena, or must not be allocated on this path).
 * Inputs are caller-owned device arrays: t1 [no][nv], t2 [no][no][nv][nv], eps [no+nv]
 * (orbital energies), ovvv [no][nv][nv][nv] = <ie|ab>, ooov [no][no][no][nv] = <jk|mc>,
 * oovv [no][no][nv][nv] = <ij|ab>; e_t is host memory.  Working memory is one static
 * 32 MiB device array per GPU: nv^3 + nv * no(no+1)(no+2)/6 doubles must fit, otherwise
 * UCC_BAD_ARGS with a message in errbuf.  Calls share that array: do not let two calls
 * overlap on the GPU.  The first call on a device looks up the array's address; make it
 * before any stream capture.  Under CUDA's lazy module loading (the default) that first
 * call is also when the device reserves the 32 MiB, so a host whose own pool claims the
 * device memory should make it before the pool does.  stream may be NULL; the call
 * returns after the result is on the host. */
ucc_status ucc_triples_noalloc(int no, int nv, const double* t1, const double* t2, const double* eps,
                               const double* ovvv, const double* ooov, const double* oovv, double* e_t,
                               void* stream, char* errbuf, size_t errlen);

/* Copy-out of named arrays: "t1" "t2" "tau" "l1" "l2" "Doo" "Dvv" "Dov" "Dvo" and the
 * HBAR blocks "Hov" "Hoo" "Hvv" "Hoooo" "Hvvvv" "Hvovv" "Hooov" "Hovvo" "Hovov" "Hvvvo"
 * "Hovoo"; per perturbation "X1:<h>" "X2:<h>" "Y1:<h>" "Y2:<h>"; "t2_guess", the T2
 * starting amplitudes the next ucc_ccsd will use (after ucc_mlp_guess or a "t2" copy-in).
 * count = elements. */
ucc_status ucc_get_tensor(ucc_ctx* ctx, const char* name, double* host_out, size_t count);
/* Copy-in (restart files, learned guesses): "t1" "t2" "l1" "l2". */
ucc_status ucc_set_tensor(ucc_ctx* ctx, const char* name, const double* host_in, size_t count);

/* ---- Learned T2 starting amplitudes (no counterpart in the reference; its guess is MP2,
 * ccwfn.cc:75-87).  A small MLP (15 pair features -> 256 -> 256 -> 1, SiLU, FP16 weights,
 * FP32 accumulation) predicts T*(t2_CCSD - t2_MP2) per doubles element, T = 1000; the
 * plain CCSD iteration started from its prediction decides the converged answer.
 * Features of element (i,j,a,b), D = e_i+e_j-e_a-e_b, S = 100: S<ij|ab>/D, S<ij|ba>/D,
 * S<ij|ab>, -1/D, (e_i+e_j)/2, (e_a+e_b)/2, [i==j], [a==b], S<ab|ab>, S<ij|ij>,
 * S(<ia|ia>+<jb|jb>), S(<ia|ai>+<jb|bj>), |e_i-e_j|/2, |e_a-e_b|/2, (e_i-e_j)(e_a-e_b)/4,
 * all invariant under (i,j,a,b) -> (j,i,b,a).  Rows are [no][no][nv][nv] order. */
typedef struct ucc_mlp ucc_mlp;
ucc_status ucc_mlp_create(ucc_mlp** net, int device, uint64_t seed);
ucc_status ucc_mlp_destroy(ucc_mlp* net);
const char* ucc_mlp_last_error(ucc_mlp* net);
int ucc_mlp_num_params(void);
/* parameters (FP32 masters) in the order W1[8][256] b1[256] W2[256][256] b2[256] w3[256] b3 */
ucc_status ucc_mlp_get_params(ucc_mlp* net, float* out, size_t count);
ucc_status ucc_mlp_set_params(ucc_mlp* net, const float* in, size_t count);
/* predictions y[rows] for features X[rows][8] (host buffers) */
ucc_status ucc_mlp_predict(ucc_mlp* net, const float* X, int64_t rows, float* y);
/* mean squared error and its gradient (count = ucc_mlp_num_params()) on one batch */
ucc_status ucc_mlp_loss_grad(ucc_mlp* net, const float* X, const float* t, int64_t rows, float* loss, float* grad,
                             size_t count);
/* Adam, minibatches of `batch` rows shuffled per epoch; final_loss = last epoch's mean */
ucc_status ucc_mlp_train(ucc_mlp* net, const float* X, const float* t, int64_t rows, int epochs, int batch, float lr,
                         uint64_t seed, float* final_loss);
/* features (and, after a converged ucc_ccsd, targets) of the loaded Hamiltonian */
ucc_status ucc_mlp_features(ucc_ctx* ctx, float* X, size_t rows, int with_targets, float* targets);
/* the next ucc_ccsd on ctx starts from t1 = f_ia/D1, t2 = t2_MP2 + prediction/T.  One
 * fused pass on the tensor cores: per 128 doubles elements the features and the first
 * layer (FP32), the second layer as a tcgen05 MMA chain (FP16 activations and weights,
 * FP32 accumulation in tensor memory) and the output layer in the epilogue; no feature
 * or activation array is written to device memory. */
ucc_status ucc_mlp_guess(ucc_ctx* ctx, ucc_mlp* net);

/* Per-stage device timings (CUDA events on the library's stream) and FLOP counts. */
/* ------------------------------------------------------------------------------------
 * Batched CCSD: many small Hamiltonians of different sizes solved together, each sweep
 * one CUDA-graph launch of grouped kernels (no counterpart in the reference, which
 * solves one molecule per call).  FP64 form; each member converges exactly as the
 * single-context solver would, and is masked out of later sweeps once it has.
 * ------------------------------------------------------------------------------------ */
typedef struct ucc_batch ucc_batch;
typedef struct ucc_batch_info {
  int members;
  int sweeps;              /* sweeps of the last solve (all of them inside one graph launch) */
  int grouped_ops;         /* recorded residual operations, each one grouped launch per sweep */
  int graph_kernels;       /* kernel nodes in the sweep graph */
  int shape_choice[4];     /* GEMM operations given tile 64x64, 32x32, 64x32, 32x64 by the autotuner */
  double solve_ms;         /* device time of the last solve (CUDA events) */
  double flops;            /* algorithmic CCSD FLOPs of the last solve, summed over members' iterations */
  double arena_bytes;      /* recorded scratch held for the members */
  int graph_launches;      /* host graph launches of the last solve (1: the sweep loop runs on the device) */
} ucc_batch_info;
ucc_status ucc_batch_create(ucc_batch** out, int device);
/* Device time limit of one ucc_batch_ccsd sweep loop (default 600 s): the loop runs on the
 * device inside a single graph launch and ends when no member is iterating, every member
 * has reached MAXITER, or this much globaltimer time has passed since the solve started;
 * the last case returns UCC_DEVICE_TIMEOUT (members keep their last amplitudes and the
 * batch stays usable). */
ucc_status ucc_batch_set_time_limit(ucc_batch* b, double seconds);
ucc_status ucc_batch_destroy(ucc_batch* b);
const char* ucc_batch_last_error(ucc_batch* b);
/* add a member from its Fock matrix [nact][nact] and factors B[naux][nact][nact] */
ucc_status ucc_batch_add_df(ucc_batch* b, int no, int nv, int naux, const double* fock, const double* B, int* index);
/* the next solve starts member `index` from the network's T2 (ucc_mlp_guess semantics) */
ucc_status ucc_batch_guess_mlp(ucc_batch* b, int index, ucc_mlp* net);
/* solve every member: e_ccsd, iterations and converged (0/1) are arrays of length members */
ucc_status ucc_batch_ccsd(ucc_batch* b, const ucc_options* opt, double* e_ccsd, int* iterations, int* converged);
ucc_status ucc_batch_get_info(ucc_batch* b, ucc_batch_info* out);
/* pair features / targets of member `index` (ucc_mlp_features semantics; targets after a
 * solve in which the member converged) */
ucc_status ucc_batch_features(ucc_batch* b, int index, float* out, size_t rows, int with_targets, float* targets);
ucc_status ucc_batch_get_t2(ucc_batch* b, int index, double* out, size_t count);

typedef struct ucc_stats {
  double ccsd_ms, triples_ms, hbar_ms, lambda_ms, density_ms, pert_ms;
  double ccsd_flops, triples_flops;
  int ccsd_iterations, lambda_iterations;
  int64_t kernel_launches;   /* kernels of this library launched since the last reset */
  double ladder_ms;          /* particle-ladder GEMM time, summed over iterations */
  double ladder_bytes;       /* its algorithmic operand bytes, summed */
  double ladder_flops;       /* its algorithmic FLOPs, summed */
  int64_t ladder_launches;
  int fp64_iterations;       /* CCSD iterations whose residual was built in FP64 */
  int64_t tc_gemm_launches;  /* tensor-core (BF16 split) GEMM launches */
  int mixed_iterations;      /* CCSD iterations with split-product residuals */
  double tc_gemm_ms;         /* device time of the tensor-core GEMMs (CUDA events) */
  double tc_gemm_flops;      /* their algorithmic FLOPs, 2*M*N*K per GEMM */
  int anchored_iterations;   /* refinement iterations built as FP64 anchor + tensor-core corrections */
  double fp64_gemm_ms;       /* device time of the FP64 GEMM launches (CUDA events) */
  double fp64_gemm_flops;    /* their algorithmic FLOPs, 2*M*N*K per GEMM */
  int64_t fp64_gemm_launches;
  double sliced_gemm_ms;     /* device time of the sliced FP64 tensor-core GEMMs (slicing included) */
  double sliced_gemm_flops;  /* their algorithmic FLOPs, 2*M*N*K per GEMM */
  int64_t sliced_gemm_launches;
  double guess_ms;           /* device time of the learned-guess pass (ucc_mlp_guess, CUDA events) */
  double sliced_gemm_product_flops; /* sliced_gemm_flops weighted by each GEMM's slice products: the tensor
                                       pipe's work (45 products per output at 9 digits, 21 at 6) */
} ucc_stats;
ucc_status ucc_get_stats(ucc_ctx* ctx, ucc_stats* out);
ucc_status ucc_reset_stats(ucc_ctx* ctx);

/* Last error message of this context (empty if none). */
const char* ucc_last_error(ucc_ctx* ctx);
const char* ucc_status_string(ucc_status s);

#ifdef __cplusplus
}
#endif
#endif /* UGACC_GB300_H */
