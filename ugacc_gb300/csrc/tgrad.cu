// (T) contributions to CCSD(T) first derivatives: tgrad_ooc of ccwfn.cc:1150-1316 (OOC=1)
// and tgrad of ccwfn.cc:854-1142 (OOC=0, the plugin's default).
//
// For every ordered occupied triple (i,j,k) the connected and disconnected triples
//   M3(abc) = W3_ijk(abc) / D3,   N3(abc) = [<ij|ab> t1_kc + <ik|ac> t1_jb + <jk|bc> t1_ia
//                                           + t2_ijab f_kc + t2_ikac f_jb + t2_jkbc f_ia] / D3
// (ccwfn.cc:1420-1454, 1492-1515) give
//   X3 = 8M(abc) - 4M(bac) - 4M(acb) - 4M(cba) + 2M(cab) + 2M(bca),  Y3 the same of N3,
//   Z3 = 2(M(abc) - M(acb)) - (M(bac) - M(bca)),  Q3 = 2 X3 + Y3,
// and the pieces
//   Dvv[a][a] += 1/2 sum_bc M3 (X3+Y3)          Dov[i][a] += sum_bc (M3 - M3(cba)) (4 t2_jkbc - 2 t2_jkcb)
//   s1[i][a]  += sum_bc (4M - 4M(bac) - 2M(acb) + 2M(cab)) <jk|bc>
//   Goovv[i][j][a][b] += 4 sum_c t1_kc Z3        X2[i][l][a][b] -= sum_c Q3 <jk|lc>
//   Gooov[j][i][l][a] -= sum_bc Q3 t2_lkbc       X2[i][j][a][d] += sum_bc Q3 <dk|bc>
//   Gvvvo[a][b][d][j] += sum_c Q3 t2_kicd        s2 = X2 + X2(ji,ba)
// The reference's second pass over (a,b,c) (:1226-1250) forms the same M3 and N3 values
// indexed by the occupied triple; because M3 and N3 are invariant under a simultaneous
// permutation of (i,j,k) and (a,b,c), its occupied-permutation X3/Y3 equal the virtual
// ones here, so Doo[i][i] -= 1/2 sum_{jk,abc} M3 (X3+Y3) reuses the Dvv partial sums.
//
// The in-core tgrad stores T3 and L3 and gives the same s1, s2, Dov, Goovv, Gooov and
// Gvvvo, and full matrices (ccwfn.cc:998-1021)
//   Doo[i][j] = -1/2 sum_{lm,def} t3_ilm^def l3_jlm^def,  Dvv[a][b] = 1/2 sum_{lmn,de} t3_lmn^bde l3_lmn^ade
// whose diagonals are the ones above: its t3 is M3 and its l3 contracts like P3 = X3 + Y3.
// With the same permutation invariance Doo[i][j] = -1/2 sum_{lm} M3_lmi . P3_lmj, so a
// batch (fixed l, a range of m, every k) adds -1/2 sum_m M3_lmk1 . P3_lmk2 to Doo[k1][k2],
// and 1/2 sum_{t,de} M3_t(bde) P3_t(ade) to Dvv[a][b]: two more engine contractions.
//
// Tuples are processed in batches (fixed i, a range of j, every k); W3 comes from the
// FP64 tuple GEMMs of the (T) energy, the element-wise work from the kernels below, and
// the four O(no^3 nv^4)-class sums from the contraction engine.  FP64, or with MIXED
// precision W3 from the tensor-core tuple GEMMs and split contractions (the pieces are
// small corrections that enter Lambda and the densities linearly).
#include <algorithm>
#include <memory>

#include "cc.h"
#include "engine.h"

namespace ucc {

void count_kernel_launch();
bool mixed_triples_batch(Ctx& c, int nbatch, const int* h_tuples, float* W3, int tblk = 0);
bool mixed_triples_prepare(Ctx& c, int max_batch);
void mixed_triples_release(Ctx& c);
void triples_operands_fp64(Ctx& c, Tensor& Acat, Tensor& Bcat);
void triples_w3_fp64(Ctx& c, const Tensor& Acat, const Tensor& Bcat, const int* h_tuples, int nb, double* W3,
                     GemmPtrs* d_ptrs);

namespace {

// W3 (FP64, or FP32 from the tensor-core tuple GEMMs: nparts partial arrays part_stride
// elements apart, W3 = their sum) -> M3; N3
template <typename TW>
__global__ void tg_prep_kernel(int no, int nv, int nt, const int* __restrict__ tuples, const TW* W, int nparts,
                               int64_t part_stride, double* M, double* N,
                               const double* __restrict__ eps, const double* __restrict__ t1,
                               const double* __restrict__ t2, const double* __restrict__ Voovv,
                               const double* __restrict__ fov) {
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv, total = (int64_t)nt * nv3;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(x / nv3);
    int64_t r = x - (int64_t)t * nv3;
    const int a = (int)(r / nv2);
    r -= (int64_t)a * nv2;
    const int b = (int)(r / nv), c = (int)(r - (int64_t)b * nv);
    const int i = tuples[3 * t], j = tuples[3 * t + 1], k = tuples[3 * t + 2];
    const double* ev = eps + no;
    double D = eps[i] + eps[j] + eps[k];
    D -= ev[a] + ev[b] + ev[c];
    const int64_t ij = ((int64_t)i * no + j) * nv2, ik = ((int64_t)i * no + k) * nv2, jk = ((int64_t)j * no + k) * nv2;
    const double num = Voovv[ij + (int64_t)a * nv + b] * t1[(int64_t)k * nv + c] +
                       Voovv[ik + (int64_t)a * nv + c] * t1[(int64_t)j * nv + b] +
                       Voovv[jk + (int64_t)b * nv + c] * t1[(int64_t)i * nv + a] +
                       t2[ij + (int64_t)a * nv + b] * fov[(int64_t)k * nv + c] +
                       t2[ik + (int64_t)a * nv + c] * fov[(int64_t)j * nv + b] +
                       t2[jk + (int64_t)b * nv + c] * fov[(int64_t)i * nv + a];
    TW w = W[x];
    for (int q = 1; q < nparts; q++) w += W[x + q * part_stride];
    M[x] = (double)w / D;
    N[x] = num / D;
  }
}

__device__ double block_sum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) / 32;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// one block per (a, tuple): Q3 and Z3 of the a-slice, and the per-(tuple, a) sums of the
// Dvv diagonal, Dov and s1 terms
__global__ void tg_reduce_kernel(int no, int nv, const int* __restrict__ tuples, const double* __restrict__ M,
                                 const double* __restrict__ N, const double* __restrict__ t2,
                                 const double* __restrict__ Voovv, double* Q, double* Z, double* P, double* pdvv,
                                 double* pdov, double* ps1) {
  const int a = blockIdx.x, t = blockIdx.y;
  const int j = tuples[3 * t + 1], k = tuples[3 * t + 2];
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv;
  const double* m = M + (int64_t)t * nv3;
  const double* n = N + (int64_t)t * nv3;
  const double* t2jk = t2 + ((int64_t)j * no + k) * nv2;
  const double* vjk = Voovv + ((int64_t)j * no + k) * nv2;
  double* q = Q + (int64_t)t * nv3 + (int64_t)a * nv2;
  double* z = Z + (int64_t)t * nv3 + (int64_t)a * nv2;
  double sdvv = 0.0, sdov = 0.0, ss1 = 0.0;
  auto at = [&](const double* A, int x, int y, int w) { return A[((int64_t)x * nv + y) * nv + w]; };
  for (int e = threadIdx.x; e < nv2; e += blockDim.x) {
    const int b = e / nv, c = e - b * nv;
    const double mabc = at(m, a, b, c), mbac = at(m, b, a, c), macb = at(m, a, c, b);
    const double mcba = at(m, c, b, a), mcab = at(m, c, a, b), mbca = at(m, b, c, a);
    const double X3 = 8.0 * mabc - 4.0 * mbac - 4.0 * macb - 4.0 * mcba + 2.0 * mcab + 2.0 * mbca;
    const double Y3 = 8.0 * at(n, a, b, c) - 4.0 * at(n, b, a, c) - 4.0 * at(n, a, c, b) - 4.0 * at(n, c, b, a) +
                      2.0 * at(n, c, a, b) + 2.0 * at(n, b, c, a);
    q[e] = 2.0 * X3 + Y3;
    z[e] = 2.0 * (mabc - macb) - (mbac - mbca);
    if (P) P[(int64_t)t * nv3 + (int64_t)a * nv2 + e] = X3 + Y3;
    sdvv += 0.5 * mabc * (X3 + Y3);
    sdov += (mabc - mcba) * (4.0 * t2jk[(int64_t)b * nv + c] - 2.0 * t2jk[(int64_t)c * nv + b]);
    ss1 += (4.0 * mabc - 4.0 * mbac - 2.0 * macb + 2.0 * mcab) * vjk[(int64_t)b * nv + c];
  }
  sdvv = block_sum(sdvv);
  sdov = block_sum(sdov);
  ss1 = block_sum(ss1);
  if (threadIdx.x == 0) {
    pdvv[(int64_t)t * nv + a] = sdvv;
    pdov[(int64_t)t * nv + a] = sdov;
    ps1[(int64_t)t * nv + a] = ss1;
  }
}

// fixed-order sums over the batch's tuples (all share the first index i)
__global__ void tg_accumulate_kernel(int no, int nv, int nt, int i, const double* __restrict__ pdvv,
                                     const double* __restrict__ pdov, const double* __restrict__ ps1, double* Dvv,
                                     double* Dov, double* s1, double* Doo) {
  double sdoo = 0.0;
  for (int a = threadIdx.x; a < nv; a += blockDim.x) {
    double dv = 0.0, dov = 0.0, s = 0.0;
    for (int t = 0; t < nt; t++) {
      dv += pdvv[(int64_t)t * nv + a];
      dov += pdov[(int64_t)t * nv + a];
      s += ps1[(int64_t)t * nv + a];
    }
    Dvv[(int64_t)a * nv + a] += dv;
    Dov[(int64_t)i * nv + a] += dov;
    s1[(int64_t)i * nv + a] += s;
    sdoo += dv;
  }
  sdoo = block_sum(sdoo);
  if (threadIdx.x == 0) Doo[(int64_t)i * no + i] -= sdoo;
}

Tensor select(const Tensor& T, int axis, int64_t idx) {  // T with one axis fixed
  Tensor r;
  r.p = T.p + idx * T.s[axis];
  r.rank = T.rank - 1;
  for (int k = 0, o = 0; k < T.rank; k++) {
    if (k == axis) continue;
    r.d[o] = T.d[k];
    r.s[o] = T.s[k];
    o++;
  }
  return r;
}

}  // namespace

void run_triples_gradient(Ctx& c) {
  UCC_REQUIRE(c.have_ccsd, UCC_BAD_STATE, "the (T) gradient needs converged CCSD amplitudes");
  const int no = c.no, nv = c.nv;
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv;
  double* T = c.get("T").p;
  Tensor t1 = amp1(c, T), t2 = amp2(c, T);
  Tensor S1 = c.alloc("TS1", {no, nv}, true);
  Tensor X2 = c.alloc("TX2", {no, no, nv, nv}, true);
  Tensor Doo = c.alloc("TDoo", {no, no}, true);
  Tensor Dvv = c.alloc("TDvv", {nv, nv}, true);
  Tensor Dov = c.alloc("TDov", {no, nv}, true);
  Tensor Goovv = c.alloc("TGoovv", {no, no, nv, nv}, true);
  Tensor Gooov = c.alloc("TGooov", {no, no, no, nv}, true);
  Tensor Gvvvo = c.alloc("TGvvvo", {nv, nv, nv, no}, true);
  // MIXED: W3 from the tensor-core tuple GEMMs (FP32 W3) and split contractions; the
  // element-wise algebra and every accumulation stay FP64
  const bool mixed = c.opt.precision == UCC_MIXED && !c.force_fp64;
  const bool full = c.opt.ooc == 0;  // in-core tgrad: full Doo and Dvv

  // batch = (fixed i, nj values of j, every k): M3, N3, Q3, Z3 of each tuple plus the
  // engine's gathered copies of Q3 / Z3
  size_t free_b = 0, total_b = 0;
  UCC_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double budget = std::min<double>(24.0e9, 0.3 * (double)free_b);
  // FP64 arrays per tuple (+ P3 and a gathered copy for the full Doo/Dvv), plus the mixed
  // form's three FP32 W3 partials (12 bytes per element)
  const double nbuf = (full ? 8.0 : 6.0) + (mixed ? 1.5 : 0.0);
  const int nj = (int)std::max<int64_t>(1, std::min<int64_t>(no, (int64_t)(budget / (nbuf * 8.0 * nv3 * no))));
  const int ntmax = nj * no;
  Tensor Acat, Bcat;
  const bool tc = mixed && mixed_triples_prepare(c, ntmax);
  if (!tc) triples_operands_fp64(c, Acat, Bcat);
  std::unique_ptr<Scratch> W32;
  // the tensor-core tuple GEMMs write W3 as three partial arrays (one per pair of terms)
  if (tc) W32 = std::make_unique<Scratch>(c, 3 * sizeof(float) * nv3 * ntmax);
  Scratch Mb(c, sizeof(double) * nv3 * ntmax), Nb(c, sizeof(double) * nv3 * ntmax);
  Scratch Qb(c, sizeof(double) * nv3 * ntmax), Zb(c, sizeof(double) * nv3 * ntmax);
  std::unique_ptr<Scratch> Pb, diag;
  if (full) {
    Pb = std::make_unique<Scratch>(c, sizeof(double) * nv3 * ntmax);
    diag = std::make_unique<Scratch>(c, sizeof(double) * ((size_t)no * no + (size_t)nv * nv));
    UCC_CUDA(cudaMemsetAsync(diag->p, 0, sizeof(double) * ((size_t)no * no + (size_t)nv * nv), c.stream));
  }
  // the diagonal sums go to TDoo/TDvv, or to a scratch copy when the full matrices are formed
  double* doo_diag = full ? diag->d() : Doo.p;
  double* dvv_diag = full ? diag->d() + (size_t)no * no : Dvv.p;
  Scratch part(c, sizeof(double) * 3 * (size_t)ntmax * nv);
  Scratch dtup(c, sizeof(int) * 3 * ntmax);
  Scratch dptr(c, sizeof(GemmPtrs) * 6 * ntmax);
  double* pdvv = part.d();
  double* pdov = pdvv + (size_t)ntmax * nv;
  double* ps1 = pdov + (size_t)ntmax * nv;
  const double* eps = c.get("eps").p;
  const double* Voovv = c.get("Voovv").p;
  const double* fov = Fk(c, "ov").p;
  Tensor Vooov = c.get("Vooov"), Vvovv = V(c, "vovv");
  std::vector<int> tuples;
  for (int i = 0; i < no; i++) {
    for (int j0 = 0; j0 < no; j0 += nj) {
      const int nb = std::min(nj, no - j0), nt = nb * no;
      tuples.clear();
      for (int j = j0; j < j0 + nb; j++)
        for (int k = 0; k < no; k++) {
          tuples.push_back(i);
          tuples.push_back(j);
          tuples.push_back(k);
        }
      UCC_CUDA(cudaMemcpyAsync(dtup.p, tuples.data(), sizeof(int) * tuples.size(), cudaMemcpyHostToDevice, c.stream));
      const int64_t total = (int64_t)nt * nv3;
      const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 32));
      if (tc) {
        mixed_triples_batch(c, nt, tuples.data(), static_cast<float*>(W32->p));
        tg_prep_kernel<float><<<g, 256, 0, c.stream>>>(no, nv, nt, static_cast<int*>(dtup.p),
                                                       static_cast<const float*>(W32->p), 3, (int64_t)nt * nv3,
                                                       Mb.d(), Nb.d(), eps, t1.p, t2.p, Voovv, fov);
      } else {
        triples_w3_fp64(c, Acat, Bcat, tuples.data(), nt, Mb.d(), static_cast<GemmPtrs*>(dptr.p));
        tg_prep_kernel<double><<<g, 256, 0, c.stream>>>(no, nv, nt, static_cast<int*>(dtup.p), Mb.d(), 1, 0,
                                                        Mb.d(), Nb.d(), eps, t1.p, t2.p, Voovv, fov);
      }
      count_kernel_launch();
      UCC_REQUIRE(nt <= 65535, UCC_BAD_ARGS, "(T) gradient: too many tuples per batch");
      tg_reduce_kernel<<<dim3((unsigned)nv, (unsigned)nt), 256, 0, c.stream>>>(
          no, nv, static_cast<int*>(dtup.p), Mb.d(), Nb.d(), t2.p, Voovv, Qb.d(), Zb.d(), full ? Pb->d() : nullptr,
          pdvv, pdov, ps1);
      count_kernel_launch();
      tg_accumulate_kernel<<<1, 256, 0, c.stream>>>(no, nv, nt, i, pdvv, pdov, ps1, dvv_diag, Dov.p, S1.p, doo_diag);
      count_kernel_launch();
      UCC_CUDA(cudaGetLastError());
      const Tensor Q = make_view(Qb.d(), {nb, no, nv, nv, nv}), Z = make_view(Zb.d(), {nb, no, nv, nv, nv});
      // Goovv[i][j][a][b] += 4 sum_kc t1[k][c] Z3
      contract(c, "jkabc,kc->jab", 4.0, Z, t1, 1.0, narrow(Goovv.slice0(i), 0, j0, nb));
      // X2[i][l][a][b] -= sum_jkc Q3 <jk|lc>
      contract(c, "jkabc,jklc->lab", -1.0, Q, narrow(Vooov, 0, j0, nb), 1.0, X2.slice0(i));
      // Gooov[j][i][l][a] -= sum_kbc Q3 t2[l][k][b][c]
      contract(c, "jkabc,lkbc->jla", -1.0, Q, t2, 1.0, select(narrow(Gooov, 0, j0, nb), 1, i));
      // X2[i][j][a][d] += sum_kbc Q3 <dk|bc>
      contract(c, "jkabc,dkbc->jad", 1.0, Q, Vvovv, 1.0, narrow(X2.slice0(i), 0, j0, nb));
      // Gvvvo[a][b][d][j] += sum_kc Q3 t2[k][i][c][d]
      contract(c, "jkabc,kcd->abdj", 1.0, Q, select(t2, 1, i), 1.0, narrow(Gvvvo, 3, j0, nb));
      if (full) {
        // Dvv[a][b] += 1/2 sum_{t,de} M3_t(bde) P3_t(ade);  Doo[k1][k2] -= 1/2 sum_{j,abc} M3_ijk1 P3_ijk2
        const Tensor M4 = make_view(Mb.d(), {nt, nv, nv, nv}), P4 = make_view(Pb->d(), {nt, nv, nv, nv});
        contract(c, "tbde,tade->ab", 0.5, M4, P4, 1.0, Dvv);
        const Tensor M3 = make_view(Mb.d(), {nb, no, nv3}), P3 = make_view(Pb->d(), {nb, no, nv3});
        contract(c, "jkx,jlx->kl", -0.5, M3, P3, 1.0, Doo);
      }
    }
  }
  // s2 = X2 + X2(ji,ba)
  Tensor S2 = c.alloc("TS2", {no, no, nv, nv}, false);
  transpose_add(c, "jiba->ijab", 1.0, X2, 0.0, S2);
  axpby(c, S2.size(), 1.0, X2.p, 1.0, S2.p);
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  c.drop("TX2");
  if (tc) {
    mixed_triples_release(c);
  } else {
    c.drop("T3_A");
    c.drop("T3_B");
  }
  c.have_tgrad = true;
}

}  // namespace ucc
