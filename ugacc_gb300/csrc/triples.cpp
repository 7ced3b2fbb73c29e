// (T) correction: the i>=j>=k W/V algorithm of ccwfn.cc:795-852 with W3_ijk (:1388-1418).
//
// W3[a,b,c] for a tuple (i,j,k) is a sum of six "e" terms (<xe|..> t2, K = nv) and six
// "m" terms (<..|mc> t2, K = no).  They pair up by output permutation, so with
//   A_x[k'][ab] = [ <xe|ab> for e ; -t2[x][m][a][b] for m ]           (nv+no) x nv^2
//   B_yz[k'][c] = [ t2[y][z][c][e] for e ; <zy|mc> for m ]           (nv+no) x nv
// every pair is one GEMM  G = A_x^T B_yz  (M = nv^2, N = nv, K = nv+no) whose epilogue
// writes G[(u,v), w] straight into W3 at the permuted position:
//   x=i (y,z)=(k,j) -> W[a][b][c]    x=i (j,k) -> W[a][c][b]    x=k (j,i) -> W[c][a][b]
//   x=k (i,j)       -> W[c][b][a]    x=j (i,k) -> W[b][c][a]    x=j (k,i) -> W[b][a][c]
// Tuples are processed in batches (one batched launch per term), then the energy kernel
// forms V3, X3, Y3, Z3 and the a>=b>=c weighted sum per tuple.
#include <algorithm>
#include <cmath>
#include <memory>

#include "cc.h"

namespace ucc {

double flops_triples(double no, double nv) { return 2.0 * no * (no + 1) * (no + 2) * nv * nv * nv * (nv + no); }

// mixed-precision tuple GEMMs (tc_gemm.cu); false if not available for this shape
bool mixed_triples_batch(Ctx& c, int nbatch, const int* h_tuples, float* W3, int tblk = 0);
bool mixed_triples_prepare(Ctx& c, int max_batch);
void mixed_triples_release(Ctx& c);

// FP64 operands: A_x (no x (nv+no) x nv^2) and B_yz (no^2 x (nv+no) x nv), as stored
// blocks "T3_A" / "T3_B" (dropped by the caller)
void triples_operands_fp64(Ctx& c, Tensor& Acat, Tensor& Bcat) {
  const int no = c.no, nv = c.nv;
  const int64_t nv2 = (int64_t)nv * nv, Kp = nv + no;
  Tensor t2 = amp2(c, c.get("T").p);
  Acat = c.alloc("T3_A", {no, Kp, nv2}, false);
  Tensor Ae = narrow(Acat, 1, 0, nv), Am = narrow(Acat, 1, nv, no);
  permute_add(c, make_view(c.get("Vovvv").p, {no, nv, nv2}), 1.0, 0.0, Ae);
  permute_add(c, make_view(t2.p, {no, no, nv2}), -1.0, 0.0, Am);
  Bcat = c.alloc("T3_B", {no, no, Kp, nv}, false);
  Tensor Be = narrow(Bcat, 2, 0, nv), Bm = narrow(Bcat, 2, nv, no);
  permute_add(c, view(t2, "yzce->yzec"), 1.0, 0.0, Be);
  permute_add(c, view(c.get("Vooov"), "zymc->yzmc"), 1.0, 0.0, Bm);
}

// W3 of nb tuples (host triples (i,j,k)) into W3 + b*nv^3, FP64; d_ptrs holds 6*nb
// pointer triples and is reused: the call synchronises before returning
void triples_w3_fp64(Ctx& c, const Tensor& Acat, const Tensor& Bcat, const int* h_tuples, int nb, double* W3,
                     GemmPtrs* d_ptrs) {
  const int no = c.no, nv = c.nv;
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv, Kp = nv + no;
  TriplesTerm terms[6];
  triples_terms(nv, terms);
  std::vector<GemmPtrs> all((size_t)nb * 6);
  for (int q = 0; q < 6; q++)
    for (int b = 0; b < nb; b++) {
      const int* ijk = h_tuples + 3 * b;
      const TriplesTerm& tm = terms[q];
      all[(size_t)q * nb + b] = {Acat.p + (int64_t)ijk[tm.x] * Kp * nv2,
                                 Bcat.p + ((int64_t)ijk[tm.y] * no + ijk[tm.z]) * Kp * nv, W3 + (int64_t)b * nv3};
    }
  UCC_CUDA(cudaMemcpyAsync(d_ptrs, all.data(), sizeof(GemmPtrs) * all.size(), cudaMemcpyHostToDevice, c.stream));
  for (int q = 0; q < 6; q++) {
    GemmEpilogue epi;
    epi.msplit = nv;
    epi.s_mhi = terms[q].su;
    epi.s_mlo = terms[q].sv;
    epi.s_n = terms[q].sw;
    dgemm_strided(c, nv2, nv, Kp, 1.0, nullptr, 1, nv2, nullptr, nv, 1, q == 0 ? 0.0 : 1.0, nullptr, epi, nb, 0, 0, 0,
                  d_ptrs + (size_t)q * nb);
  }
  // the pointer array is reused by the next batch: keep the copy ordered after use
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

double run_triples(Ctx& c) {
  UCC_REQUIRE(c.have_ccsd, UCC_BAD_STATE, "(T) needs converged CCSD amplitudes");
  const int no = c.no, nv = c.nv;
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv;
  double* T = c.get("T").p;
  Tensor t1 = amp1(c, T);

  std::vector<int> tuples;
  for (int i = 0; i < no; i++)
    for (int j = 0; j <= i; j++)
      for (int k = 0; k <= j; k++) {
        tuples.push_back(i);
        tuples.push_back(j);
        tuples.push_back(k);
      }
  const int ntup = (int)tuples.size() / 3;
  size_t free_b = 0, total_b = 0;
  UCC_CUDA(cudaMemGetInfo(&free_b, &total_b));
  // larger batches let more tuples that share an A operand read it from L2 (the batched
  // GEMM walks its tiles M-group-major across the batch)
  const double budget = std::min<double>(24.0e9, 0.25 * (double)free_b);
  // W3 bytes per tuple: FP64, or three FP32 partial arrays (one per pair of terms) in the
  // mixed form
  const bool want_mixed = c.opt.precision == UCC_MIXED && !c.force_fp64;
  // nv % 4 == 0: the pipelined energy kernel, which reads W3 in 8 x 8 x 8 blocks
  // (w3_block_offset; nv rounded up to whole blocks; the GEMM epilogue addresses a tuple's
  // blocks with 32-bit offsets, so up to 2^31 floats per tuple, nv <= 1288)
  const int64_t tb = (nv + 7) / 8;
  const int tblk = want_mixed && nv % 4 == 0 && tb * tb * tb * 512 < ((int64_t)1 << 31) ? (int)tb : 0;
  const int64_t w3_per = tblk ? (int64_t)tblk * tblk * tblk * 512 : nv3;  // elements per tuple and array
  const double w3_bytes = (want_mixed ? 12.0 : 8.0) * (double)w3_per;
  const int batch = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)(budget / w3_bytes), 4096, ntup}));

  Scratch dtup(c, sizeof(int) * tuples.size());
  UCC_CUDA(cudaMemcpyAsync(dtup.p, tuples.data(), sizeof(int) * tuples.size(), cudaMemcpyHostToDevice, c.stream));
  Scratch W3(c, (size_t)std::ceil(w3_bytes) * batch);
  const bool mixed = want_mixed && mixed_triples_prepare(c, batch);
  // per-tuple partial sums: one per virtual index a (FP64 kernel) or per virtual tile triple (FP32)
  const int64_t pstride = mixed ? triples_f32_partials(nv) : nv;
  Scratch partial(c, sizeof(double) * (size_t)ntup * pstride);

  // FP64 path: concatenated operands A_x and B_yz
  Tensor Acat, Bcat;
  if (!mixed) triples_operands_fp64(c, Acat, Bcat);
  // mixed path: FP32 copies of the energy's integral inputs (pipelined energy kernel)
  std::unique_ptr<Scratch> f32in;
  if (mixed && tblk) {
    f32in = std::make_unique<Scratch>(c, sizeof(float) * (size_t)triples_f32_layout(no, nv).total);
    triples_f32_inputs(c, no, nv, t1.p, c.get("Voovv").p, c.get("eps").p, static_cast<float*>(f32in->p));
  }
  Scratch dptr(c, sizeof(GemmPtrs) * batch * 6);
  GemmPtrs* dp = static_cast<GemmPtrs*>(dptr.p);
  for (int t0 = 0; t0 < ntup; t0 += batch) {
    const int nb = std::min(batch, ntup - t0);
    if (mixed)
      mixed_triples_batch(c, nb, tuples.data() + 3 * t0, static_cast<float*>(W3.p), f32in ? tblk : 0);
    else
      triples_w3_fp64(c, Acat, Bcat, tuples.data() + 3 * t0, nb, W3.d(), dp);
    if (mixed)
      triples_energy_f32(c, no, nv, nb, static_cast<int*>(dtup.p) + 3 * t0, static_cast<const float*>(W3.p), 3,
                         (int64_t)nb * (f32in ? w3_per : nv3), t1.p, c.get("Voovv").p, c.get("eps").p,
                         partial.d() + (int64_t)t0 * pstride, f32in ? static_cast<const float*>(f32in->p) : nullptr);
    else
      triples_energy(c, no, nv, nb, static_cast<int*>(dtup.p) + 3 * t0, W3.d(), t1.p, c.get("Voovv").p,
                     c.get("eps").p, partial.d() + (int64_t)t0 * nv);
  }
  Scratch et(c, sizeof(double));
  dot_async(c, (int64_t)ntup * pstride, partial.d(), nullptr, et.d());
  double e = 0.0;
  UCC_CUDA(cudaMemcpyAsync(&e, et.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  if (mixed) {
    mixed_triples_release(c);
  } else {
    c.drop("T3_A");
    c.drop("T3_B");
  }
  tc_check(c);
  UCC_REQUIRE(std::isfinite(e), UCC_NAN_DETECTED, "(T) energy is not finite");
  return e;
}

}  // namespace ucc
