// (T) energy from caller-owned device buffers, with no device allocation at all.
//
// Some host programs cannot let a library call cudaMalloc: applications that hand all
// device memory to their own arena/pool allocator and account for every byte, code that
// runs while another component holds the memory budget, or callers on a path where an
// allocation could stall or fail at a bad moment.  ucc_triples_noalloc serves them: the
// caller passes every input and output, and the only working memory is the fixed
// file-scope device array below, which every GPU that loads this library keeps until the
// process exits.
//
// Limits and sharing rules:
//  * the working set (nv^3 doubles for one tuple's W3 block plus nv doubles per i>=j>=k
//    occupied triple) must fit in kScratchDoubles (32 MiB); larger problems are rejected
//    with UCC_BAD_ARGS and a message;
//  * all calls share the array and it keeps the last call's contents; every element a
//    call reads is written earlier in that same call, so nothing needs clearing, but two
//    calls whose work overlaps on the GPU (different streams, or several host threads)
//    race on it and must not be issued;
//  * the first call on a device looks up the array's device address with that device
//    current (cudaGetSymbolAddress) and caches it; make that first call before any
//    stream capture.  With CUDA's lazy module loading (the default) that first call is
//    also when the 32 MiB are reserved on the device, so a host whose own pool takes the
//    device memory should make it before the pool does;
//  * a call whose stream is not capturing looks the address up again (cheap), so the
//    cached value never outlives a cudaDeviceReset or a module reload.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/ugacc_gb300.h"

namespace {

constexpr size_t kScratchDoubles = (size_t)32 << 17;  // 4 Mi doubles = 32 MiB

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;

void put_msg(char* buf, size_t len, const char* msg) {
  if (buf && len) {
    std::strncpy(buf, msg, len - 1);
    buf[len - 1] = '\0';
  }
}

// W3[a][b][c] of ccwfn.cc:1388-1418 for one (i,j,k), one thread per (a,b,c)
__global__ void w3_direct_kernel(int no, int nv, int i, int j, int k, const double* t2, const double* ovvv,
                                 const double* ooov, double* W) {
  const int64_t nv2 = (int64_t)nv * nv, nv3 = nv2 * nv;
  const int64_t nvo = (int64_t)no * nv;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nv3; x += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(x % nv), b = (int)((x / nv) % nv), a = (int)(x / nv2);
    // <pe|qr> with p occupied: ovvv[p][e][q][r]; t2[p][q][r][s]
    auto V = [&](int p, int e, int q, int r) { return ovvv[((int64_t)p * nv + e) * nv2 + (int64_t)q * nv + r]; };
    auto T = [&](int p, int q, int r, int s) { return t2[((int64_t)p * no + q) * nv2 + (int64_t)r * nv + s]; };
    auto O = [&](int p, int q, int m, int r) { return ooov[((int64_t)p * no + q) * nvo + (int64_t)m * nv + r]; };
    double v = 0.0;
    for (int e = 0; e < nv; e++)
      v += V(i, e, a, b) * T(k, j, c, e) + V(i, e, a, c) * T(j, k, b, e) + V(k, e, c, a) * T(j, i, b, e) +
           V(k, e, c, b) * T(i, j, a, e) + V(j, e, b, c) * T(i, k, a, e) + V(j, e, b, a) * T(k, i, c, e);
    for (int m = 0; m < no; m++)
      v -= O(j, k, m, c) * T(i, m, a, b) + O(k, j, m, b) * T(i, m, a, c) + O(i, j, m, b) * T(k, m, c, a) +
           O(j, i, m, a) * T(k, m, c, b) + O(k, i, m, a) * T(j, m, b, c) + O(i, k, m, c) * T(j, m, b, a);
    W[x] = v;
  }
}

// energy contribution of one tuple (ccwfn.cc:813-849), one block per a; partial[a]
__global__ void tuple_energy_kernel(int no, int nv, int i, int j, int k, const double* W, const double* t1,
                                    const double* oovv, const double* eps, double* partial) {
  __shared__ double sh[32];
  const int a = blockIdx.x;
  const int64_t nv2 = (int64_t)nv * nv;
  const double* Vij = oovv + ((int64_t)i * no + j) * nv2;
  const double* Vik = oovv + ((int64_t)i * no + k) * nv2;
  const double* Vjk = oovv + ((int64_t)j * no + k) * nv2;
  const double eijk = eps[i] + eps[j] + eps[k];
  const double fac = 2.0 - (double)((i == j) + (i == k) + (j == k));
  double s = 0.0;
  for (int q = threadIdx.x; q < (a + 1) * (a + 1); q += blockDim.x) {
    const int b = q / (a + 1), c = q % (a + 1);
    if (c > b) continue;
    auto Wv = [&](int x, int y, int z) { return W[(int64_t)x * nv2 + (int64_t)y * nv + z]; };
    auto Vv = [&](int x, int y, int z) {
      return (Wv(x, y, z) + Vij[(int64_t)x * nv + y] * t1[(int64_t)k * nv + z] +
              Vik[(int64_t)x * nv + z] * t1[(int64_t)j * nv + y] + Vjk[(int64_t)y * nv + z] * t1[(int64_t)i * nv + x]) /
             (1.0 + (double)((x == y) + (x == z) + (y == z)));
    };
    const double wabc = Wv(a, b, c), wacb = Wv(a, c, b), wbac = Wv(b, a, c);
    const double wbca = Wv(b, c, a), wcab = Wv(c, a, b), wcba = Wv(c, b, a);
    const double vabc = Vv(a, b, c), vacb = Vv(a, c, b), vbac = Vv(b, a, c);
    const double vbca = Vv(b, c, a), vcab = Vv(c, a, b), vcba = Vv(c, b, a);
    const double X3 = wabc * vabc + wacb * vacb + wbac * vbac + wbca * vbca + wcab * vcab + wcba * vcba;
    const double Y3 = vabc + vbca + vcab, Z3 = vacb + vbac + vcba;
    const double d3 = eijk - (eps[no + a] + eps[no + b] + eps[no + c]);
    s += ((Y3 - 2.0 * Z3) * (wabc + wbca + wcab) + (Z3 - 2.0 * Y3) * (wacb + wbac + wcba) + 3.0 * X3) * fac / d3;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); w++) t += sh[w];
    partial[a] = t;
  }
}

// compensated sum of n partials, one block
__global__ void sum_partials_kernel(int64_t n, const double* x, double* out) {
  __shared__ double sh[256];
  double s = 0.0, c = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double t = s + x[i];
    c += (fabs(s) >= fabs(x[i])) ? (s - t) + x[i] : (x[i] - t) + s;
    s = t;
  }
  sh[threadIdx.x] = s + c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0, cc = 0.0;
    for (int r = 0; r < (int)blockDim.x; r++) {
      const double t = tot + sh[r];
      cc += (fabs(tot) >= fabs(sh[r])) ? (tot - t) + sh[r] : (sh[r] - t) + tot;
      tot = t;
    }
    *out = tot + cc;
  }
}

}  // namespace

extern "C" ucc_status ucc_triples_noalloc(int no, int nv, const double* t1, const double* t2, const double* eps,
                                          const double* ovvv, const double* ooov, const double* oovv, double* e_t,
                                          void* stream, char* errbuf, size_t errlen) {
  if (no < 1 || nv < 1 || !t1 || !t2 || !eps || !ovvv || !ooov || !oovv || !e_t) {
    put_msg(errbuf, errlen, "ucc_triples_noalloc: need no, nv >= 1 and non-null pointers");
    return UCC_BAD_ARGS;
  }
  const size_t nv3 = (size_t)nv * nv * nv;
  const size_t ntup = (size_t)no * (no + 1) * (no + 2) / 6;
  const size_t need = nv3 + ntup * (size_t)nv + 1;
  if (need > kScratchDoubles) {
    char m[256];
    std::snprintf(m, sizeof m,
                  "ucc_triples_noalloc: no=%d nv=%d needs %zu doubles of working memory, the static scratch holds %zu "
                  "(32 MiB); use ucc_triples for larger systems",
                  no, nv, need, kScratchDoubles);
    put_msg(errbuf, errlen, m);
    return UCC_BAD_ARGS;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    put_msg(errbuf, errlen, "ucc_triples_noalloc: no current CUDA device");
    return UCC_CUDA_ERROR;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    // once per device, with that device current; again on every call outside a stream
    // capture, so that a reset device (a reloaded module) gets its new address
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t qrc = cudaStreamIsCapturing(st, &cap);
    if (qrc != cudaSuccess) cudaGetLastError();  // the failed query's error is not left behind
    const bool capturing = qrc != cudaSuccess || cap != cudaStreamCaptureStatusNone;
    if (!g_scratch_ptr[dev] || !capturing) {
      void* p = nullptr;
      const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (rc != cudaSuccess || !p) {
        put_msg(errbuf, errlen, cudaGetErrorString(rc));
        return UCC_CUDA_ERROR;
      }
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  double* W = scratch;
  double* partial = scratch + nv3;
  double* total = partial + ntup * nv;
  const unsigned wblocks = (unsigned)((nv3 + 255) / 256 < 4096 ? (nv3 + 255) / 256 : 4096);
  size_t t = 0;
  for (int i = 0; i < no; i++)
    for (int j = 0; j <= i; j++)
      for (int k = 0; k <= j; k++, t++) {
        w3_direct_kernel<<<wblocks, 256, 0, st>>>(no, nv, i, j, k, t2, ovvv, ooov, W);
        tuple_energy_kernel<<<nv, 256, 0, st>>>(no, nv, i, j, k, W, t1, oovv, eps, partial + t * nv);
      }
  sum_partials_kernel<<<1, 256, 0, st>>>((int64_t)(ntup * nv), partial, total);
  cudaError_t rc = cudaGetLastError();
  if (rc == cudaSuccess) rc = cudaMemcpyAsync(e_t, total, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (rc == cudaSuccess) rc = cudaStreamSynchronize(st);
  if (rc != cudaSuccess) {
    put_msg(errbuf, errlen, cudaGetErrorString(rc));
    return UCC_CUDA_ERROR;
  }
  put_msg(errbuf, errlen, "");
  return UCC_OK;
}
