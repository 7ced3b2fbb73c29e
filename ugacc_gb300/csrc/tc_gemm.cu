// Mixed-precision tensor-core GEMM for sm_103a (tcgen05 + TMEM + TMA).
//
// C[m][n] (FP64, strided, alpha/beta, permuting epilogue) =
//     sum_k  Ahi[m][k] Bhi[n][k] + Ahi[m][k] Blo[n][k] + Alo[m][k] Bhi[n][k]
// where x = hi + lo with hi = bf16(x), lo = bf16(x - hi): the two-term split product of
// FP64 operands, accumulated in FP32 in tensor memory.  The three products are one
// K loop over 3 * K/64 blocks that switches the TMA source between the hi and lo copies.
//
// Kernel layout (one CTA per SM, persistent over 128 x 256 output tiles):
//   warp 0      TMA producer (one thread): A 128x64 and B 256x64 bf16 tiles, 128B swizzle
//   warp 1      MMA issuer (one thread): tcgen05.mma.cta_group::1.kind::f16, M=128 N=256 K=16
//   warps 2-5   epilogue: tcgen05.ld 32x32b.x32 -> FP64 alpha/beta -> global
//   4-stage smem ring (full/empty mbarriers), two TMEM accumulators (2 x 256 columns) so
//   the epilogue of one tile overlaps the MMAs of the next.
// Every mbarrier wait is bounded (globaltimer deadline); on expiry the kernel raises a
// device error flag, the other warps see it and leave their loops, TMEM is released and
// the host reports UCC_DEVICE_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstring>
#include <map>
#include <tuple>

#include "cc.h"
#include "core.h"
#include "tc_ptx.h"

namespace ucc {

void count_kernel_launch();  // kernels_fp64.cu
// C(epi) = alpha * sum_z P[z] + beta * C(epi) (kernels_fp64.cu)
void splitk_reduce(Ctx& c, int64_t M, int64_t N, int nsplit, const double* P, double alpha, double beta, double* C,
                   const GemmEpilogue& epi);

namespace tc {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4, THREADS = 192;
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
constexpr uint32_t TMEM_COLS = 2 * BN;
constexpr size_t SMEM_BYTES = 1024 + (size_t)STAGES * (A_BYTES + B_BYTES) + 256;
// N tile for N output columns: the fewest tiles of at most 256 columns, each a multiple of
// 32 (N = 320 takes two tiles of 160 rather than 256 + 64)
inline int pick_bn(int64_t N) {
  const int64_t nt = (N + 255) / 256;
  return (int)(((N + nt - 1) / nt + 31) / 32 * 32);
}
// CTAs per cluster for a launch with mtiles M tiles: pairs that share the B tile whenever
// there are two M tiles to pair (the B maps then have boxes of bn / 2 rows)
inline int cluster_m(int mtiles) { return mtiles >= 2 ? 2 : 1; }

// gemm_kernel: an operand ring of 216 KB (four 48 KB stages, or fused stages of
// A_hi | A_lo | B_hi | B_lo), then the barriers
constexpr size_t GEMM_RING = 216 * 1024;
constexpr size_t GEMM_SMEM_BYTES = 1024 + GEMM_RING + 256;
// instruction descriptor, kind::f16: D f32 (bit 4), A bf16 (bits 7-9 = 1), B bf16
// (bits 10-12 = 1), both K-major, N>>3 at bits 17-22, M>>4 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

struct Params {
  int M, N, kblocks, mtiles, ntiles;
  int bn;  // N tile: the MMA's N and the B box rows (a multiple of 32 up to 256)
  double alpha, beta;
  double* C;
  GemmEpilogue epi;
  int* err;
  // batched problems of one shape (0 = a single problem): problem p reads A rows from
  // a_row0[p] and B rows from b_row0[p] of the tensor maps and writes C + c_off[p]
  int nprob;
  const int* a_row0;
  const int* b_row0;
  const int64_t* c_off;
  // split-K (single problem only): chunk z covers K blocks [z*kchunk, (z+1)*kchunk) of each
  // of the three split products and writes a plain [M][N] FP64 partial at C + z*M*N
  int ksplit, kchunk;
  // nterms = 2 (batched problems only): a second product accumulated into the same tile,
  // A from the second pair of tensor maps at rows a_row1[p], B at rows b_row1[p]
  int nterms;
  const int* a_row1;
  const int* b_row1;
  // C32 != null: FP32 output C32[off] = alpha * acc (+ C32[off] when beta != 0), no FP64
  // work in the epilogue (GB300 issues ~4 FP64 operations per clock per SM)
  float* C32;
  // nparts = 3: operands split hi + mid + lo (third maps), six products hi.hi, hi.mid,
  // mid.hi, hi.lo, mid.mid, lo.hi (representation error ~2^-25 instead of ~2^-17)
  int nparts;
  // kc > 0: the K range of every tile runs in chunks of kc K blocks, each chunk's FP32
  // accumulator added into the FP64 output by the epilogue (the first with beta, the
  // rest with 1), which bounds the FP32 accumulation chain; FP64 output only
  int kc;
  // fused (two parts, kc == 0): one ring stage holds A_hi, A_lo, B_hi and B_lo of a K block
  // and the three products are issued from it (a third less operand traffic than one
  // stage per product); nst stages of stage_bytes each
  int fused, nst, stage_bytes;
  // tblk > 0 (FP32 output of the (T) tuple GEMMs, alpha 1, beta 0): W3 in the blocked
  // layout of w3_block_offset with tblk blocks per index; the strides s_mhi, s_mlo, s_n
  // (nv^2, nv or 1, msplit = nv) say which of a, b, c each index is
  int tblk = 0;
};

// v[p] <- v[p ^ k] for 0 <= k < 8: three conditional swaps (selects, no indexed registers)
__device__ __forceinline__ void xor_swap8(float (&v)[8], int k) {
#pragma unroll
  for (int bit = 1; bit < 8; bit <<= 1) {
    const bool s = (k & bit) != 0;
#pragma unroll
    for (int e = 0; e < 8; e++)
      if ((e & bit) == 0) {
        const float lo = v[e], hi = v[e | bit];
        v[e] = s ? hi : lo;
        v[e | bit] = s ? lo : hi;
      }
  }
}

// the split products of one K block: (A part, B part), part 0 = hi, 1 = lo (2 parts) or
// 0 = hi, 1 = mid, 2 = lo (3 parts)
__device__ __forceinline__ void seg_parts(int nparts, int seg, int& pa, int& pb) {
  if (nparts == 3) {  // A parts 0,0,1,0,1,2 and B parts 0,1,0,2,1,0, two bits per segment
    pa = (2320 >> (2 * seg)) & 3;
    pb = (388 >> (2 * seg)) & 3;
  } else {
    pa = seg == 2 ? 1 : 0;
    pb = seg == 1 ? 1 : 0;
  }
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc));
}
// N tiles per raster band: the tiles of one problem run band by band, and inside a band M
// group by M group with the band's N tiles fastest, so that the ~150 tiles in flight at a
// time cover about a dozen M groups x RASTER_N N tiles: each A tile is then read by
// RASTER_N concurrent tiles and each B tile by a dozen, mostly from L2 (walking M fastest
// over a whole column of tiles shared B only and re-read every A tile from DRAM once per N
// tile).
constexpr int RASTER_N = 8;
__device__ __forceinline__ void raster(int mgroups, int ntiles, int tl, int& mg, int& nt) {
  const int band = tl / (mgroups * RASTER_N);
  const int w = min(RASTER_N, ntiles - band * RASTER_N);  // N tiles in this band
  const int r = tl - band * mgroups * RASTER_N;
  mg = r / w;
  nt = band * RASTER_N + (r - mg * w);
}

// Work item -> (problem or K chunk pb, M tile group mg, N tile nt).  Batched problems run
// M-group-major: all problems and N tiles of one M group before the next, so that the
// problems of a launch that share an A operand (the (T) tuples of one occupied index) read
// each A tile from L2 instead of DRAM.  One problem (or its split-K chunks) runs
// chunk-major, each chunk in raster bands.
__device__ __forceinline__ void tile_coords(const Params& p, int mgroups, int tile, int& pb, int& mg, int& nt) {
  if (p.nprob) {
    const int per_m = p.nprob * p.ntiles;
    mg = tile / per_m;
    const int r = tile - mg * per_m;
    pb = r / p.ntiles;
    nt = r - pb * p.ntiles;
  } else {
    const int tiles_per = mgroups * p.ntiles;
    pb = tile / tiles_per;
    raster(mgroups, p.ntiles, tile - pb * tiles_per, mg, nt);
  }
}

// CM CTAs per cluster along M (1 or 2).  With CM = 2 the two CTAs of a cluster take M tiles
// 2j and 2j+1 of the same N tile: each loads half of the B tile's rows and multicasts it
// into both CTAs' rings (the B tensor maps have boxes of bn / 2 rows), so every B byte
// crosses from L2 once per pair; a ring stage is refilled only after the MMAs of both CTAs
// released it (each MMA commit arrives on the stage's empty barrier in both CTAs).
template <int CM>
__global__ void __launch_bounds__(THREADS, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                const __grid_constant__ CUtensorMap mA2hi, const __grid_constant__ CUtensorMap mA2lo,
                const __grid_constant__ CUtensorMap mAmid, const __grid_constant__ CUtensorMap mBmid, Params p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_BYTES;
  uint64_t* full = (uint64_t*)(smem + GEMM_RING);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* mdone = tempty + 2;  // every MMA of this CTA has completed (before TMEM is released)
  uint32_t* tslot = (uint32_t*)(mdone + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nst = p.fused ? p.nst : STAGES;  // ring stages (at most STAGES)
  const int rank = CM > 1 ? (int)cluster_rank() : 0;
  constexpr uint16_t kMask = (uint16_t)((1u << CM) - 1u);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CM);  // released by the MMAs of every CTA that reads the multicast B
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], 128);
    }
    mbar_init(mdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (CM > 1) cluster_sync();  // the peer's barriers exist before its multicasts or arrivals reach them
  const uint32_t tmem = *tslot;
  // M tiles in groups of CM (one per CTA of the cluster); the clusters walk the groups
  const int mgroups = (p.mtiles + CM - 1) / CM;
  const int tiles_per = mgroups * p.ntiles;
  const int ntile = tiles_per * (p.nprob ? p.nprob : (p.ksplit > 1 ? p.ksplit : 1));
  const int cid = blockIdx.x / CM, ncl = gridDim.x / CM;
  const int bh = p.bn / CM;  // B rows this CTA loads (for every CTA of the cluster)
  // ring items per K block and term: one fused stage, or one stage per split product
  const int nseg = p.fused ? 1 : (p.nparts == 3 ? 6 : 3);
  const uint32_t b_tile = (uint32_t)(p.bn * BK * 2);
  // K chunks of one tile (in-kernel chunking) and the K blocks of chunk ch
  const int nch = p.kc > 0 ? (p.kblocks + p.kc - 1) / p.kc : 1;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t issued = 0;
      bool ok = true;
      for (int tile = cid; tile < ntile && ok; tile += ncl) {
        int pb, mg, nt;
        tile_coords(p, mgroups, tile, pb, mg, nt);
        const int mt = mg * CM + rank;
        const int ar0 = (p.nprob ? p.a_row0[pb] : 0) + mt * BM;
        const int br0 = (p.nprob ? p.b_row0[pb] : 0) + nt * p.bn + rank * bh;
        const int ar1 = p.nterms > 1 ? p.a_row1[pb] + mt * BM : 0;
        const int br1 = p.nterms > 1 ? p.b_row1[pb] + nt * p.bn + rank * bh : 0;
        for (int ch = 0; ch < nch && ok; ch++) {
          int k0 = 0, kn = p.kblocks;
          if (p.ksplit > 1) {
            k0 = pb * p.kchunk;
            kn = min(p.kblocks - k0, p.kchunk);
          } else if (p.kc > 0) {
            k0 = ch * p.kc;
            kn = min(p.kblocks - k0, p.kc);
          }
          for (int kb = 0; kb < p.nterms * nseg * kn; kb++) {
            if (!mbar_wait(&empty[stage], phase ^ 1u, p.err)) {
              ok = false;
              break;
            }
            const int term = kb / (nseg * kn), w = kb - term * nseg * kn;
            const int seg = w / kn, kk = (k0 + w - seg * kn) * BK;
            // this CTA's share of the B tile (all of it when CM = 1) goes to every CTA of the cluster
            auto load_b = [&](uint8_t* dst, const CUtensorMap* map, int row) {
              if (CM == 1)
                tma_load(dst, map, &full[stage], kk, row);
              else
                tma_load_mc(dst + (size_t)rank * bh * BK * 2, map, &full[stage], kk, row, kMask);
            };
            if (p.fused) {  // A_hi | A_lo | B_hi | B_lo of K block kk
              uint8_t* st = smem + (size_t)stage * p.stage_bytes;
              mbar_expect_tx(&full[stage], (uint32_t)(2 * A_BYTES) + 2 * b_tile);
              tma_load(st, term == 0 ? &mAhi : &mA2hi, &full[stage], kk, term == 0 ? ar0 : ar1);
              tma_load(st + A_BYTES, term == 0 ? &mAlo : &mA2lo, &full[stage], kk, term == 0 ? ar0 : ar1);
              load_b(st + 2 * A_BYTES, &mBhi, term == 0 ? br0 : br1);
              load_b(st + 2 * A_BYTES + b_tile, &mBlo, term == 0 ? br0 : br1);
            } else {
              int pa, pbp;
              seg_parts(p.nparts, seg, pa, pbp);
              const CUtensorMap* ma = term == 0 ? (pa == 0 ? &mAhi : (pa == 1 && p.nparts == 3) ? &mAmid : &mAlo)
                                                : (pa == 0 ? &mA2hi : &mA2lo);
              const CUtensorMap* mb = pbp == 0 ? &mBhi : (pbp == 1 && p.nparts == 3) ? &mBmid : &mBlo;
              mbar_expect_tx(&full[stage], (uint32_t)A_BYTES + b_tile);
              tma_load(sA + stage * A_BYTES, ma, &full[stage], kk, term == 0 ? ar0 : ar1);
              load_b(sB + stage * B_BYTES, mb, term == 0 ? br0 : br1);
            }
            ++issued;
            if (++stage == nst) {
              stage = 0;
              phase ^= 1u;
            }
          }
        }
      }
      // the last ring loads must have landed before the CTA may exit (matters only on an
      // error path; normally the epilogue's final wait already implies it)
      for (int64_t n = issued > nst ? issued - nst : 0; n < issued; n++)
        mbar_wait_deadline(&full[n % nst], (uint32_t)((n / nst) & 1));
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0, acc = 0;
      uint32_t phase = 0, aphase = 0;
      bool ok = true;
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(p.bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      for (int tile = cid; tile < ntile && ok; tile += ncl) {
        for (int ch = 0; ch < nch && ok; ch++) {
          int kn = p.kblocks;
          if (p.ksplit > 1)
            kn = min(p.kblocks - (tile / tiles_per) * p.kchunk, p.kchunk);
          else if (p.kc > 0)
            kn = min(p.kblocks - ch * p.kc, p.kc);
          if (!mbar_wait(&tempty[acc], aphase ^ 1u, p.err)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t d = tmem + (uint32_t)(acc * BN);
          for (int kb = 0; kb < p.nterms * nseg * kn; kb++) {
            if (!mbar_wait(&full[stage], phase, p.err)) {
              ok = false;
              break;
            }
            fence_after();
            if (p.fused) {  // hi.hi, hi.lo, lo.hi from one stage
              uint8_t* st = smem + (size_t)stage * p.stage_bytes;
              const uint64_t ahi = sdesc(st), alo = sdesc(st + A_BYTES);
              const uint64_t bhi = sdesc(st + 2 * A_BYTES), blo = sdesc(st + 2 * A_BYTES + b_tile);
#pragma unroll
              for (int pr = 0; pr < 3; pr++) {
                const uint64_t ad = pr == 2 ? alo : ahi, bd = pr == 1 ? blo : bhi;
#pragma unroll
                for (int k = 0; k < BK / 16; k++)
                  mma_i(d, ad + (uint64_t)(k * 2), bd + (uint64_t)(k * 2), idesc, (kb | pr | k) != 0);
              }
            } else {
              const uint64_t ad = sdesc(sA + stage * A_BYTES), bd = sdesc(sB + stage * B_BYTES);
#pragma unroll
              for (int k = 0; k < BK / 16; k++)  // +32 bytes along K per 16-element step
                mma_i(d, ad + (uint64_t)(k * 2), bd + (uint64_t)(k * 2), idesc, (kb | k) != 0);
            }
            if (CM == 1)
              mma_commit(&empty[stage]);
            else
              mma_commit_mc(&empty[stage], kMask);  // the stage is free here and in the peer
            if (++stage == nst) {
              stage = 0;
              phase ^= 1u;
            }
          }
          mma_commit(&tfull[acc]);
          if (++acc == 2) {
            acc = 0;
            aphase ^= 1u;
          }
        }
      }
      // on an error path the loop may end with MMAs still running: wait for all of them
      // before the CTA releases tensor memory
      mma_commit(mdone);
      mbar_wait_deadline(mdone, 0);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    int acc = 0;
    uint32_t aphase = 0;
    const GemmEpilogue ep = p.epi;
    bool ok = true;
    for (int tile = cid; tile < ntile && ok; tile += ncl)
    for (int kch = 0; kch < nch; kch++) {
      int pb, mg, nt;
      tile_coords(p, mgroups, tile, pb, mg, nt);
      const int mt = mg * CM + rank;
      const int64_t coff = p.nprob ? p.c_off[pb] : (p.ksplit > 1 ? (int64_t)pb * p.M * p.N : 0);
      if (!mbar_wait(&tfull[acc], aphase, p.err)) {
        ok = false;
        break;
      }
      fence_after();
      const int64_t m = (int64_t)mt * BM + q * 32 + lane;
      const int64_t mo = ep.msplit ? (m / ep.msplit) * ep.s_mhi + (m % ep.msplit) * ep.s_mlo : m * ep.s_mhi;
      // later K chunks of a tile add onto the earlier ones
      const double alpha = p.alpha, beta = kch == 0 ? p.beta : 1.0;
      for (int ch = 0; ch < p.bn / 32; ch++) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + ch * 32), r);
        if (m < p.M) {
          const int64_t n0 = (int64_t)nt * p.bn + ch * 32;
          // with beta != 0 all 32 old values are loaded before the first store, so the
          // loads are in flight together instead of each waiting behind a store that
          // might alias it
          if (p.C32 && p.tblk) {
            // blocked W3: each index placed by its linear stride (nv^2 a, nv b, 1 c)
            const int64_t nvv = ep.msplit, hi = m / nvv, lo = m % nvv, T = p.tblk;
            const int rn = ep.s_n == 1 ? 2 : (ep.s_n == nvv ? 1 : 0);
            const int rh = ep.s_mhi == 1 ? 2 : (ep.s_mhi == nvv ? 1 : 0);
            float* Cw = p.C32 + coff;
            if (rn == 2 && n0 + 32 <= p.N) {
              // the 32 columns are c: four 8-wide c blocks, each a contiguous 32 bytes
              // holding element z at z ^ k, stored as two float4 after the same swap
              const int64_t a = rh == 0 ? hi : lo, b = rh == 0 ? lo : hi;
              const int x = (int)(a & 7), y = (int)(b & 7), k = (5 * y) & 7;
              float* base = Cw + (((a >> 3) * T + (b >> 3)) * T) * 512 + 64 * x + 8 * (y ^ x);
#pragma unroll
              for (int g = 0; g < 4; g++) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; e++) v[e] = __uint_as_float(r[8 * g + e]);
                xor_swap8(v, k);
                float4* dst = reinterpret_cast<float4*>(base + ((n0 >> 3) + g) * 512);
                dst[0] = make_float4(v[0], v[1], v[2], v[3]);
                dst[1] = make_float4(v[4], v[5], v[6], v[7]);
              }
            } else {
              // the 32 columns are four 8-wide blocks of one index (n0 % 32 == 0): the
              // offset is a block part, linear in the block, plus one of eight in-block
              // offsets fixed by the row (32-bit: a tuple's blocks hold < 2^31 floats)
              const int rl = 3 - rn - rh;
              const int fa = (int)(rh == 0 ? hi : (rl == 0 ? lo : 0)), fb = (int)(rh == 1 ? hi : (rl == 1 ? lo : 0));
              const int fc = (int)(rh == 2 ? hi : (rl == 2 ? lo : 0)), nb0 = (int)(n0 >> 3), Ti = (int)T;
              const int bA = rn == 0 ? nb0 : fa >> 3, bB = rn == 1 ? nb0 : fb >> 3, bC = rn == 2 ? nb0 : fc >> 3;
              const int blk0 = ((bA * Ti + bB) * Ti + bC) * 512;
              const int gstride = (rn == 0 ? Ti * Ti : (rn == 1 ? Ti : 1)) * 512;
              int loc[8];
#pragma unroll
              for (int e = 0; e < 8; e++) {
                const int x = rn == 0 ? e : (fa & 7), y = rn == 1 ? e : (fb & 7), z = rn == 2 ? e : (fc & 7);
                loc[e] = 64 * x + 8 * (y ^ x) + (z ^ ((5 * y) & 7));
              }
#pragma unroll
              for (int j = 0; j < 32; j++)
                if (n0 + j < p.N) Cw[blk0 + (j >> 3) * gstride + loc[j & 7]] = __uint_as_float(r[j]);
            }
          } else if (p.C32) {
            float* Cf = p.C32 + coff + mo;
            const float af = (float)alpha;
            if (ep.s_n == 1 && beta == 0.0 && af == 1.0f && n0 + 32 <= p.N &&
                ((reinterpret_cast<uintptr_t>(Cf + n0) & 15u) == 0)) {
              // a lane's 32 columns are contiguous: 16-byte stores, 8 per lane instead of 32
              float4* dst = reinterpret_cast<float4*>(Cf + n0);
#pragma unroll
              for (int j = 0; j < 8; j++)
                dst[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                                     __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
            } else {
              float old[32];
#pragma unroll
              for (int j = 0; j < 32; j++) old[j] = (beta != 0.0 && n0 + j < p.N) ? Cf[(n0 + j) * ep.s_n] : 0.f;
#pragma unroll
              for (int j = 0; j < 32; j++)
                if (n0 + j < p.N) Cf[(n0 + j) * ep.s_n] = fmaf(af, __uint_as_float(r[j]), old[j]);
            }
          } else if (alpha == 1.0 && (beta == 0.0 || beta == 1.0)) {
            double* Cb = p.C + coff + mo;
            double old[32];
#pragma unroll
            for (int j = 0; j < 32; j++) old[j] = (beta != 0.0 && n0 + j < p.N) ? Cb[(n0 + j) * ep.s_n] : 0.0;
#pragma unroll
            for (int j = 0; j < 32; j++)
              if (n0 + j < p.N) Cb[(n0 + j) * ep.s_n] = old[j] + f32_bits_to_f64(r[j]);
          } else {
            double* Cb = p.C + coff + mo;
#pragma unroll
            for (int j = 0; j < 32; j++) {
              const int64_t n = n0 + j;
              if (n < p.N) {
                double* cp = Cb + n * ep.s_n;
                const double v = alpha * (double)__uint_as_float(r[j]);
                *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
              }
            }
          }
        }
      }
      fence_before();
      mbar_arrive(&tempty[acc]);
      if (++acc == 2) {
        acc = 0;
        aphase ^= 1u;
      }
    }
  }
  fence_before();
  __syncthreads();
  // no CTA leaves while its peer may still multicast into its ring or arrive on its barriers
  if (CM > 1) cluster_sync();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// ------------------------------------------------------------------------------------
// FP64 GEMM from exact BF16 slices (the error-free splitting of Ozaki, Ogita, Oishi and
// Rump, Numer. Algorithms 59 (2012) 95-118, with base-2^SB digits, SB = 6).
//
// Every operand row r is scaled by 2^-e_r (e_r = ilogb(max_k |x_rk|) + 2, so the scaled
// row lies in (-1/2, 1/2)) and written as S balanced base-2^SB digits,
//   x_rk = 2^e_r sum_{s<S} d_s(r,k) 2^-SB(s+1),  |d_s| <= 2^(SB-1) = 32,
// stored pre-scaled as bf16 slices d_s 2^-SB(s+1) (exact: small integers times a power of
// two).  A product of an A slice s and a B slice t is an integer times 2^-SB(s+t+2), at most
// 2^10 in magnitude, so any sum of up to 2^14 such products with the same s+t is exact in
// the FP32 tensor-memory accumulator.  The kernel therefore accumulates, per output tile,
// "units": for each order g = s+t < gex, every pair (s, g-s) over a K range of at most
// 2^14 / (g+1) elements (exact), and one tail unit with all pairs of order gex..S-1 over the
// whole K range (FP32, its terms are ~2^-SB gex smaller than the leading ones).  The
// epilogue adds each unit into the FP64 output as
//   C[m][n] += alpha 2^(e_m + e_n) acc,
// the first unit of a tile applying beta.  Pairs with s+t >= S are dropped (truncation
// ~2^-SB S relative to max|A_m.| max|B_.n|).  Fewer, wider digits (SB = 7) would need 20 %
// fewer products but 4x more units, and the global read-modify-write of every unit's
// epilogue is what limits this kernel.
// ------------------------------------------------------------------------------------
struct SParams {
  int M, N, kblocks, mtiles, ntiles;
  int bn;              // N tile (a multiple of 32 up to 256): the MMA's N and the B box rows
  int S, gex;          // slices per operand; orders below gex are accumulated exactly
  int a_rows, b_rows;  // rows per slice in the slice arrays (slice s of row r at s * rows + r)
  double alpha, beta;
  double* C;
  GemmEpilogue epi;
  const int* ea;  // row exponents of A and B
  const int* eb;
  int* err;
  int ksplit, kchunk;  // split-K into FP64 partials at C + z*M*N (alpha 1, beta 0)
};

struct SUnit {
  int g0, g1, kb0, kb1;  // orders [g0, g1], K blocks [kb0, kb1)
};

constexpr int SB = 6;                                           // bits per digit
constexpr int kSlices = 9;  // digits per operand of the full-precision product (9 x 6 = 54 bits)
constexpr int SEXACT_KB = (1 << (24 - 2 * (SB - 1))) / BK;     // K blocks of one pair per exact unit

// K blocks per exact unit of order g: (g+1) pairs x kc blocks x 64 <= 2^(24 - 2(SB-1)) products
__device__ __forceinline__ int sunit_kc(int g) { return max(1, SEXACT_KB / (g + 1)); }

__device__ __forceinline__ int sunit_count(int S, int gex, int kn) {
  int u = gex < S ? 1 : 0;
  for (int g = 0; g < gex; g++) {
    const int kc = sunit_kc(g);
    u += (kn + kc - 1) / kc;
  }
  return u;
}

__device__ __forceinline__ SUnit sunit_at(int S, int gex, int k0, int kn, int u) {
  for (int g = 0; g < gex; g++) {
    const int kc = sunit_kc(g), nu = (kn + kc - 1) / kc;
    if (u < nu) return SUnit{g, g, k0 + u * kc, k0 + min((u + 1) * kc, kn)};
    u -= nu;
  }
  return SUnit{gex, S - 1, k0, k0 + kn};
}

__device__ __forceinline__ int sunit_items(const SUnit& U) {
  int pairs = 0;
  for (int g = U.g0; g <= U.g1; g++) pairs += g + 1;
  return pairs * (U.kb1 - U.kb0);
}

__device__ __forceinline__ double pow2i(int e) {  // 2^e for -1022 <= e <= 1023
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// shared memory of the sliced kernel: the operand ring, barriers, and a 32 x 33 FP32
// transpose buffer per epilogue warp
constexpr size_t SLICED_SMEM_BYTES = SMEM_BYTES + 4 * 32 * 33 * sizeof(float);

// CM = 2: as gemm_kernel<2>, the two CTAs of a cluster take neighbouring M tiles and each
// multicasts half of every B slice tile into both rings.
template <int CM>
__global__ void __launch_bounds__(THREADS, 1)
    sliced_gemm_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, SParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_BYTES;
  uint64_t* full = (uint64_t*)(sB + STAGES * B_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* mdone = tempty + 2;  // every MMA of this CTA has completed (before TMEM is released)
  uint32_t* tslot = (uint32_t*)(mdone + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int rank = CM > 1 ? (int)cluster_rank() : 0;
  constexpr uint16_t kMask = (uint16_t)((1u << CM) - 1u);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CM);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], 128);
    }
    mbar_init(mdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (CM > 1) cluster_sync();
  const uint32_t tmem = *tslot;
  const int mgroups = (p.mtiles + CM - 1) / CM;
  const int tiles_per = mgroups * p.ntiles;
  const int ntile = tiles_per * (p.ksplit > 1 ? p.ksplit : 1);
  const int cid = blockIdx.x / CM, ncl = gridDim.x / CM;
  const int bh = p.bn / CM;
  // K range of a tile: the whole K, or chunk z of a split-K launch
  auto krange = [&](int tile, int& k0, int& kn) {
    k0 = 0;
    kn = p.kblocks;
    if (p.ksplit > 1) {
      k0 = (tile / tiles_per) * p.kchunk;
      kn = min(p.kblocks - k0, p.kchunk);
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t issued = 0;
      bool ok = true;
      for (int tile = cid; tile < ntile && ok; tile += ncl) {
        int mg, ntl;
        raster(mgroups, p.ntiles, tile % tiles_per, mg, ntl);
        const int m0 = (mg * CM + rank) * BM, n0 = ntl * p.bn + rank * bh;
        int k0, kn;
        krange(tile, k0, kn);
        const int nu = sunit_count(p.S, p.gex, kn);
        for (int u = 0; u < nu && ok; u++) {
          const SUnit U = sunit_at(p.S, p.gex, k0, kn, u);
          for (int g = U.g0; g <= U.g1 && ok; g++)
            for (int s = 0; s <= g && ok; s++)
              for (int kb = U.kb0; kb < U.kb1; kb++) {
                if (!mbar_wait(&empty[stage], phase ^ 1u, p.err)) {
                  ok = false;
                  break;
                }
                mbar_expect_tx(&full[stage], (uint32_t)(A_BYTES + p.bn * BK * 2));
                tma_load(sA + stage * A_BYTES, &mA, &full[stage], kb * BK, s * p.a_rows + m0);
                if (CM == 1)
                  tma_load(sB + stage * B_BYTES, &mB, &full[stage], kb * BK, (g - s) * p.b_rows + n0);
                else
                  tma_load_mc(sB + stage * B_BYTES + (size_t)rank * bh * BK * 2, &mB, &full[stage], kb * BK,
                              (g - s) * p.b_rows + n0, kMask);
                ++issued;
                if (++stage == STAGES) {
                  stage = 0;
                  phase ^= 1u;
                }
              }
        }
      }
      for (int64_t n = issued > STAGES ? issued - STAGES : 0; n < issued; n++)
        mbar_wait_deadline(&full[n % STAGES], (uint32_t)((n / STAGES) & 1));
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0, acc = 0;
      uint32_t phase = 0, aphase = 0;
      bool ok = true;
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(p.bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      for (int tile = cid; tile < ntile && ok; tile += ncl) {
        int k0, kn;
        krange(tile, k0, kn);
        const int nu = sunit_count(p.S, p.gex, kn);
        for (int u = 0; u < nu && ok; u++) {
          const int items = sunit_items(sunit_at(p.S, p.gex, k0, kn, u));
          if (!mbar_wait(&tempty[acc], aphase ^ 1u, p.err)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t d = tmem + (uint32_t)(acc * BN);
          for (int kb = 0; kb < items; kb++) {
            if (!mbar_wait(&full[stage], phase, p.err)) {
              ok = false;
              break;
            }
            fence_after();
            const uint64_t ad = sdesc(sA + stage * A_BYTES), bd = sdesc(sB + stage * B_BYTES);
#pragma unroll
            for (int k = 0; k < BK / 16; k++)
              mma_i(d, ad + (uint64_t)(k * 2), bd + (uint64_t)(k * 2), idesc, (kb | k) != 0);
            if (CM == 1)
              mma_commit(&empty[stage]);
            else
              mma_commit_mc(&empty[stage], kMask);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1u;
            }
          }
          mma_commit(&tfull[acc]);
          if (++acc == 2) {
            acc = 0;
            aphase ^= 1u;
          }
        }
      }
      mma_commit(mdone);  // as in gemm_kernel: no MMA in flight when TMEM is released
      mbar_wait_deadline(mdone, 0);
    }
  } else {
    const int q = warp & 3;
    int acc = 0;
    uint32_t aphase = 0;
    const GemmEpilogue ep = p.epi;
    bool ok = true;
    const int nch = p.bn / 32;
    for (int tile = cid; tile < ntile && ok; tile += ncl) {
      int mg, nt;
      raster(mgroups, p.ntiles, tile % tiles_per, mg, nt);
      const int mt = mg * CM + rank;
      const int64_t coff = p.ksplit > 1 ? (int64_t)(tile / tiles_per) * p.M * p.N : 0;
      int k0, kn;
      krange(tile, k0, kn);
      const int nu = sunit_count(p.S, p.gex, kn);
      const int64_t mw = (int64_t)mt * BM + q * 32;  // first row of this warp
      const int64_t m = mw + lane;
      auto moff = [&](int64_t mm) {
        return ep.msplit ? (mm / ep.msplit) * ep.s_mhi + (mm % ep.msplit) * ep.s_mlo : mm * ep.s_mhi;
      };
      const int64_t mo = moff(m);
      // alpha 2^e_m; the column factor 2^e_n is added to its exponent field (|e| <= 500 and
      // 2^-20 <= |alpha| <= 2^20 keep the result normal)
      const long long sa = m < p.M ? __double_as_longlong(p.alpha * pow2i(p.ea[m])) : 0;
      // lanes run along the rows when those are contiguous in C; otherwise the 32 x 32 block
      // is transposed through shared memory so that lanes run along the columns
      const bool rows_contiguous = ep.msplit == 0 && ep.s_mhi == 1;
      float* tsm = reinterpret_cast<float*>(smem + STAGES * (A_BYTES + B_BYTES) + 256) + (warp - 2) * 32 * 33;
      for (int u = 0; u < nu; u++) {
        if (!mbar_wait(&tfull[acc], aphase, p.err)) {
          ok = false;
          break;
        }
        fence_after();
        const bool first = u == 0;
        const bool load_old = !(first && p.beta == 0.0);
        for (int ch = 0; ch < nch; ch++) {
          uint32_t r[32];
          tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + ch * 32), r);
          const int64_t n0 = (int64_t)nt * p.bn + ch * 32;
          if (rows_contiguous) {
            if (m < p.M) {
              double* Cb = p.C + coff + mo;
#pragma unroll
              for (int h = 0; h < 32; h += 16) {  // 16 columns at a time: loads in flight together
                double old[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                  old[j] = 0.0;
                  if (n0 + h + j < p.N && load_old) {
                    old[j] = Cb[(n0 + h + j) * ep.s_n];
                    if (first) old[j] *= p.beta;
                  }
                }
#pragma unroll
                for (int j = 0; j < 16; j++)
                  if (n0 + h + j < p.N) {
                    const double f = __longlong_as_double(sa + ((long long)p.eb[n0 + h + j] << 52));
                    Cb[(n0 + h + j) * ep.s_n] = fma(f32_bits_to_f64(r[h + j]), f, old[j]);
                  }
              }
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; j++) tsm[lane * 33 + j] = __uint_as_float(r[j]);
            __syncwarp();
            const int64_t n = n0 + lane;  // this lane's column
            const bool nok = n < p.N;
            const long long ebs = nok ? (long long)p.eb[n] << 52 : 0;
            double* Cn = p.C + coff + n * ep.s_n;
#pragma unroll
            for (int h = 0; h < 32; h += 16) {
              double old[16];
#pragma unroll
              for (int i = 0; i < 16; i++) {
                old[i] = 0.0;
                if (nok && mw + h + i < p.M && load_old) {
                  old[i] = Cn[moff(mw + h + i)];
                  if (first) old[i] *= p.beta;
                }
              }
#pragma unroll
              for (int i = 0; i < 16; i++) {
                const long long sai = __shfl_sync(0xffffffffu, sa, h + i);
                if (nok && mw + h + i < p.M)
                  Cn[moff(mw + h + i)] = fma(f32_bits_to_f64(__float_as_uint(tsm[(h + i) * 33 + lane])),
                                             __longlong_as_double(sai + ebs), old[i]);
              }
            }
            __syncwarp();
          }
        }
        fence_before();
        mbar_arrive(&tempty[acc]);
        if (++acc == 2) {
          acc = 0;
          aphase ^= 1u;
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (CM > 1) cluster_sync();  // the peer no longer multicasts into this ring
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// element (r, k) of a two-stride operand view (r, k and the splits below 2^32: 32-bit division)
__device__ __forceinline__ const double& mv_at(const MatView& v, int64_t r, int64_t k) {
  int64_t ro = r * v.rs_hi, ko = k * v.ks_hi;
  if (v.rsplit) {
    const uint32_t q = (uint32_t)r / (uint32_t)v.rsplit;
    ro = (int64_t)q * v.rs_hi + ((int64_t)r - (int64_t)q * v.rsplit) * v.rs_lo;
  }
  if (v.ksplit) {
    const uint32_t q = (uint32_t)k / (uint32_t)v.ksplit;
    ko = (int64_t)q * v.ks_hi + ((int64_t)k - (int64_t)q * v.ksplit) * v.ks_lo;
  }
  return v.p[ro + ko];
}
__device__ __forceinline__ bool mv_kcontig(const MatView& v) { return (v.ksplit ? v.ks_lo : v.ks_hi) == 1; }

// row maxima |x| of a rows x cols FP64 view as bit patterns (non-negative doubles order
// like their bits, so the maximum is an integer one); block (x, y) covers 32 rows and the
// K range [x kchunk, (x+1) kchunk), lanes along k (sk == 1) or along the rows (transposed
// views), and merges into amax (zeroed by the caller) with one atomicMax per row
__global__ void slice_absmax_kernel(MatView x, int64_t kchunk, unsigned long long* amax) {
  __shared__ unsigned long long t[8][32];
  const int64_t rows = x.rows, cols = x.cols;
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * kchunk;
  const int64_t k1 = min(cols, k0 + kchunk);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const unsigned long long absmask = 0x7FFFFFFFFFFFFFFFull;
  if (mv_kcontig(x)) {
    for (int i = ty; i < 32; i += 8) {
      const int64_t r = r0 + i;
      unsigned long long mm = 0;
      if (r < rows)
        for (int64_t k = k0 + tx; k < k1; k += 32)
          mm = max(mm, (unsigned long long)__double_as_longlong(mv_at(x, r, k)) & absmask);
      for (int o = 16; o > 0; o >>= 1) mm = max(mm, __shfl_xor_sync(0xffffffffu, mm, o));
      if (tx == 0 && r < rows && mm) atomicMax(amax + r, mm);
    }
  } else {
    const int64_t r = r0 + tx;
    unsigned long long mm = 0;
    if (r < rows)
      for (int64_t k = k0 + ty; k < k1; k += 8)
        mm = max(mm, (unsigned long long)__double_as_longlong(mv_at(x, r, k)) & absmask);
    t[ty][tx] = mm;
    __syncthreads();
    if (ty == 0 && r < rows) {
      for (int i = 1; i < 8; i++) mm = max(mm, t[i][tx]);
      if (mm) atomicMax(amax + r, mm);
    }
  }
}

// row exponent from the row maximum: e = ilogb(max) + 2 (max/2^e in [1/4, 1/2)), clamped
// below at -500; a row maximum >= 2^498 sets *range (the caller falls back to FP64)
__device__ __forceinline__ int slice_exponent(unsigned long long bits, int* range) {
  const int be = (int)((bits >> 52) & 0x7FF);
  if (be == 0) return -500;  // zero or subnormal row maximum
  const int e = be - 1023 + 2;
  if (e > 500) {
    atomicExch(range, 1);
    return 500;
  }
  return max(e, -500);
}

// x 2^(bits-e) rounded to an integer (|result| < 2^(bits-1) since |x| < 2^(e-1); bits <= 56),
// from the bit fields of x with integer operations only
__device__ __forceinline__ long long slice_fixed(double x, int e, int bits) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FF);
  const long long mant = (long long)(b & 0xFFFFFFFFFFFFFull) | (E ? (1ll << 52) : 0ll);
  const int shift = max(E, 1) - 1075 + bits - e;  // x = mant 2^(max(E,1) - 1075)
  long long v;
  if (shift >= 0)
    v = mant << shift;
  else if (shift > -63)
    v = (mant + (1ll << (-shift - 1))) >> (-shift);
  else
    v = 0;
  return (b >> 63) ? -v : v;
}

// digits: slices[s][r][k] = bf16(d_s 2^-SB(s+1)) for r < rows_p (zero past rows), k < kp
// (zero past cols), the balanced base-2^SB digits of x 2^(SB S - e) (least significant s = S-1);
// e[r] written by the blocks of the first K tile.  32 x 64 tiles through shared memory:
// reads coalesced along whichever stride is 1; each thread then slices two neighbouring
// elements of a row and stores each digit pair as one bf16x2 (a warp writes 128
// contiguous bytes of a slice plane per store; kp is a multiple of 64).
__global__ void slice_digits_kernel(MatView x, int64_t rows_p, int64_t kp, const unsigned long long* __restrict__ amax,
                                    int S, __nv_bfloat16* slices, int* e_out, int* range) {
  __shared__ double t[32][65];
  const int64_t rows = x.rows, cols = x.cols;
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 64;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (mv_kcontig(x)) {
    for (int i = ty; i < 32; i += 8)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int64_t r = r0 + i, k = k0 + tx + 32 * h;
        t[i][tx + 32 * h] = (r < rows && k < cols) ? mv_at(x, r, k) : 0.0;
      }
  } else {
    for (int j = ty; j < 64; j += 8) {
      const int64_t r = r0 + tx, k = k0 + j;
      t[tx][j] = (r < rows && k < cols) ? mv_at(x, r, k) : 0.0;
    }
  }
  __syncthreads();
  const size_t plane2 = (size_t)rows_p * kp / 2;  // a slice plane in bf16 pairs
  constexpr int H = 1 << (SB - 1);
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i, k = k0 + 2 * tx;
    if (r >= rows_p) continue;
    const int e = r < rows ? slice_exponent(amax[r], range) : 0;
    if (k == 0 && r < rows) e_out[r] = e;
    long long X0 = r < rows ? slice_fixed(t[i][2 * tx], e, SB * S) : 0;
    long long X1 = r < rows ? slice_fixed(t[i][2 * tx + 1], e, SB * S) : 0;
    __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(slices + (size_t)r * kp + k);
    // digit s (|d| <= 2^(SB-1)): a 32-bit conversion, exact, and exact in bf16 after the
    // power-of-2 scale
    auto put = [&](int s, int d0, int d1) {
      const float sc = __int_as_float((127 - SB * (s + 1)) << 23);
      dst[(size_t)s * plane2] = __floats2bfloat162_rn((float)d0 * sc, (float)d1 * sc);
    };
    if (S >= 6) {
      // balanced digits in 32-bit arithmetic: the low 30 bits hold the 5 least significant
      // digits, whose carry out (0 or 1) joins the high part for the other S - 5
      int lo0 = (int)(X0 & 0x3FFFFFFFll), hi0 = (int)(X0 >> 30);
      int lo1 = (int)(X1 & 0x3FFFFFFFll), hi1 = (int)(X1 >> 30);
      int s = S - 1;
      for (int q = 0; q < 5; q++, s--) {
        const int d0 = ((lo0 + H) & (2 * H - 1)) - H, d1 = ((lo1 + H) & (2 * H - 1)) - H;  // in [-H, H)
        lo0 = (lo0 - d0) >> SB;
        lo1 = (lo1 - d1) >> SB;
        put(s, d0, d1);
      }
      hi0 += lo0;
      hi1 += lo1;
      for (; s > 0; s--) {
        const int d0 = ((hi0 + H) & (2 * H - 1)) - H, d1 = ((hi1 + H) & (2 * H - 1)) - H;
        hi0 = (hi0 - d0) >> SB;
        hi1 = (hi1 - d1) >> SB;
        put(s, d0, d1);
      }
      put(0, hi0, hi1);  // what remains: |d| <= H
    } else {
      for (int s = S - 1; s >= 0; s--) {
        long long d0, d1;
        if (s > 0) {
          d0 = ((X0 + H) & (2 * H - 1)) - H;  // balanced digit in [-H, H)
          d1 = ((X1 + H) & (2 * H - 1)) - H;
          X0 = (X0 - d0) >> SB;
          X1 = (X1 - d1) >> SB;
        } else {
          d0 = X0;  // what remains: |d| <= H
          d1 = X1;
        }
        put(s, (int)d0, (int)d1);
      }
    }
  }
}

// FP64 rows x cols view (strides sr, sk) -> bf16 hi/lo [rows][kp], zero padded to kp
// (mid != null: three parts, x = hi + mid + lo, each the bf16 rounding of what remains)
// 32 x 64 tiles through shared memory: reads coalesced along whichever stride is 1 (sk == 1:
// along k, otherwise along the rows); each thread splits two neighbouring elements of a row
// and stores each part as one bf16x2 (128 contiguous bytes per warp store; kp is a
// multiple of 64).  Two parts are formed in FP32 (x truncated to FP32 first, from its bit
// fields: 2^-23, far below the lo part's 2^-17), three parts in FP64.
__global__ void split_kernel(MatView x, int64_t kp, __nv_bfloat16* hi, __nv_bfloat16* lo, __nv_bfloat16* mid) {
  __shared__ double t[32][65];
  const int64_t rows = x.rows, cols = x.cols;
  const int64_t k0 = (int64_t)blockIdx.x * 64;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool kc = mv_kcontig(x);
  for (int64_t r0 = (int64_t)blockIdx.y * 32; r0 < rows; r0 += (int64_t)gridDim.y * 32) {  // row tiles
  __syncthreads();
  if (kc) {
    for (int i = ty; i < 32; i += 8)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int64_t r = r0 + i, k = k0 + tx + 32 * h;
        t[i][tx + 32 * h] = (r < rows && k < cols) ? mv_at(x, r, k) : 0.0;
      }
  } else {
    for (int j = ty; j < 64; j += 8) {
      const int64_t r = r0 + tx, k = k0 + j;
      t[tx][j] = (r < rows && k < cols) ? mv_at(x, r, k) : 0.0;
    }
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i, k = k0 + 2 * tx;
    if (r >= rows) continue;
    const int64_t o2 = (r * kp + k) / 2;  // bf16 pair index
    const double v0 = t[i][2 * tx], v1 = t[i][2 * tx + 1];
    if (mid) {
      const __nv_bfloat16 h0 = __double2bfloat16(v0), h1 = __double2bfloat16(v1);
      double r0d = v0 - (double)__bfloat162float(h0), r1d = v1 - (double)__bfloat162float(h1);
      const __nv_bfloat16 m0 = __double2bfloat16(r0d), m1 = __double2bfloat16(r1d);
      r0d -= (double)__bfloat162float(m0);
      r1d -= (double)__bfloat162float(m1);
      reinterpret_cast<__nv_bfloat162*>(hi)[o2] = __halves2bfloat162(h0, h1);
      reinterpret_cast<__nv_bfloat162*>(mid)[o2] = __halves2bfloat162(m0, m1);
      reinterpret_cast<__nv_bfloat162*>(lo)[o2] = __halves2bfloat162(__double2bfloat16(r0d), __double2bfloat16(r1d));
    } else {
      const float f0 = f64_to_f32_trunc(v0), f1 = f64_to_f32_trunc(v1);
      const __nv_bfloat16 h0 = __float2bfloat16_rn(f0), h1 = __float2bfloat16_rn(f1);
      reinterpret_cast<__nv_bfloat162*>(hi)[o2] = __halves2bfloat162(h0, h1);
      reinterpret_cast<__nv_bfloat162*>(lo)[o2] =
          __halves2bfloat162(__float2bfloat16_rn(f0 - __bfloat162float(h0)), __float2bfloat16_rn(f1 - __bfloat162float(h1)));
    }
  }
  }
}

// The bounded-wait path of the pipelines above, exercised on its own: thread 0 waits, with
// the same mbar_wait and the given limit, on a barrier that nothing arrives on, so the wait
// runs out, raises the error flag and the kernel returns; the host then sees the flag
// exactly as after a stalled GEMM pipeline.
__global__ void wait_selftest_kernel(int* err, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait(&bar, 0, err, limit_ns);
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
struct Split {
  __nv_bfloat16* hi = nullptr;
  __nv_bfloat16* lo = nullptr;
  __nv_bfloat16* mid = nullptr;  // three-part splits only
  std::unique_ptr<Scratch> tmp;  // storage of a temporary (non-constant) operand
  int64_t rows = 0, kp = 0;
  CUtensorMap mhi, mlo, mmid;  // tensor maps of the last box_rows asked for (maps_for)
  int map_rows = 0;
  ~Split() {
    if (tmp) return;
    if (hi) cudaFree(hi);
    if (lo) cudaFree(lo);
    if (mid) cudaFree(mid);
  }
};

// an operand as S exact bf16 slices [S][rows_p][kp] with row exponents (sliced FP64 GEMM)
struct Sliced {
  __nv_bfloat16* d = nullptr;
  int* e = nullptr;
  std::unique_ptr<Scratch> tmp;  // storage of a temporary (non-constant) operand
  int64_t rows = 0, rows_p = 0, kp = 0;
  int S = 0;
  CUtensorMap map;  // for boxes of map_rows rows (slice_map)
  int map_rows = 0;
  ~Sliced() {
    if (!tmp) {
      if (d) cudaFree(d);
      if (e) cudaFree(e);
    }
  }
};

// an operand of the caches: the view (pointer, shape, strides), the box rows and the parts
using Key = std::tuple<const double*, int64_t, int64_t, int64_t, int64_t, int64_t, int64_t, int64_t, int64_t, int, int>;
static Key make_key(const MatView& v, int box_rows, int parts) {
  return Key{v.p, v.rows, v.cols, v.rsplit, v.rs_hi, v.rs_lo, v.ksplit, v.ks_hi, v.ks_lo, box_rows, parts};
}
struct Triples;
struct Cache {
  std::map<Key, std::unique_ptr<Split>> ops;
  std::map<Key, std::unique_ptr<Sliced>> sliced;
  int* range = nullptr;    // device flag: a sliced operand row maximum beyond the range (sticky)
  int* pinned = nullptr;   // host copies of err and range, refreshed in stream order after launches
  bool sattr_set = false;
  int max_pairs_sliced = 0;  // clusters of two sliced_gemm_kernel CTAs resident at once
  std::shared_ptr<Triples> triples;
  int* err = nullptr;
  int sms = 0;
  bool attr_set = false;
  int max_pairs = 0;  // clusters of two gemm_kernel CTAs resident at once
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~Cache() {
    if (err) cudaFree(err);  // err and range share one allocation
    if (pinned) cudaFreeHost(pinned);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    UCC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
    UCC_REQUIRE(q == cudaDriverEntryPointSuccess && f, UCC_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
    fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  }
  return fn;
}

static void make_map(CUtensorMap* m, void* base, int64_t rows, int64_t kp, int box_rows) {
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  UCC_REQUIRE(r == CUDA_SUCCESS, UCC_CUDA_ERROR, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

static Cache& cache(Ctx& c) {
  if (!c.tc_cache) {
    auto* k = new Cache;
    c.tc_cache = std::shared_ptr<void>(k, [](void* p) { delete static_cast<Cache*>(p); });
    UCC_CUDA(cudaMalloc(&k->err, 2 * sizeof(int)));
    UCC_CUDA(cudaMemset(k->err, 0, 2 * sizeof(int)));
    k->range = k->err + 1;
    UCC_CUDA(cudaMallocHost(&k->pinned, 2 * sizeof(int)));
    k->pinned[0] = k->pinned[1] = 0;
    UCC_CUDA(cudaDeviceGetAttribute(&k->sms, cudaDevAttrMultiProcessorCount, c.device));
    UCC_CUDA(cudaEventCreate(&k->ev0));
    UCC_CUDA(cudaEventCreate(&k->ev1));
  }
  return *static_cast<Cache*>(c.tc_cache.get());
}

// the operand's tensor maps for boxes of box_rows x 64
static Split* maps_for(Split* s, int box_rows, int parts) {
  if (s->map_rows != box_rows) {
    make_map(&s->mhi, s->hi, s->rows, s->kp, box_rows);
    make_map(&s->mlo, s->lo, s->rows, s->kp, box_rows);
    if (parts == 3) make_map(&s->mmid, s->mid, s->rows, s->kp, box_rows);
    s->map_rows = box_rows;
  }
  return s;
}

// split (and cache when the source is a constant block) a rows x cols FP64 operand
static Split* prepare(Ctx& c, const MatView& x, int box_rows, std::unique_ptr<Split>& temp, int parts = 2) {
  Cache& k = cache(c);
  const bool constant = c.is_constant(x.p);
  const int64_t rows = x.rows, cols = x.cols;
  UCC_REQUIRE(rows < INT32_MAX && cols < INT32_MAX, UCC_BAD_ARGS, "tensor-core GEMM: operand too large");
  // the split data does not depend on the box a launch reads it with (maps_for)
  const Key key = make_key(x, 0, parts);
  if (constant) {
    auto it = k.ops.find(key);
    if (it != k.ops.end()) return maps_for(it->second.get(), box_rows, parts);
  }
  auto s = std::make_unique<Split>();
  s->rows = rows;
  s->kp = (cols + BK - 1) / BK * BK;
  const size_t plane = sizeof(__nv_bfloat16) * rows * s->kp;  // a multiple of 128 bytes
  if (constant) {
    UCC_CUDA(cudaMalloc(&s->hi, plane));
    UCC_CUDA(cudaMalloc(&s->lo, plane));
    if (parts == 3) UCC_CUDA(cudaMalloc(&s->mid, plane));
  } else {  // stream-ordered pool: no device synchronisation per temporary
    s->tmp = std::make_unique<Scratch>(c, plane * (parts == 3 ? 3 : 2));
    s->hi = static_cast<__nv_bfloat16*>(s->tmp->p);
    s->lo = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(s->tmp->p) + plane);
    if (parts == 3) s->mid = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(s->tmp->p) + 2 * plane);
  }
  split_kernel<<<dim3((unsigned)(s->kp / 64), (unsigned)std::min<int64_t>((rows + 31) / 32, 65535)), dim3(32, 8), 0,
                 c.stream>>>(x, s->kp, s->hi, s->lo, s->mid);
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
  maps_for(s.get(), box_rows, parts);
  Split* raw = s.get();
  if (constant)
    k.ops[key] = std::move(s);
  else
    temp = std::move(s);
  return raw;
}

// the slices' tensor map for boxes of box_rows x 64
static Sliced* slice_map(Sliced* s, int box_rows) {
  if (s->map_rows != box_rows) {
    make_map(&s->map, s->d, (int64_t)s->S * s->rows_p, s->kp, box_rows);
    s->map_rows = box_rows;
  }
  return s;
}

// slice (and cache when the source is a constant block and memory allows) a rows x cols
// FP64 operand; the slice arrays are padded to whole tiles of pad_rows rows so that no tile
// reaches into the next slice, and read with boxes of box_rows rows (pad_rows or a half).
// A cached operand always holds all kSlices digits: a product with S < kSlices digits reads
// the leading S of them (they differ from x by less than one unit of digit S-1, like an
// S-digit split).  nullptr when the slices do not fit in free memory.
static Sliced* slice_prepare(Ctx& c, const MatView& x, int pad_rows, int box_rows, int S,
                             std::unique_ptr<Sliced>& temp, bool allow_cache) {
  Cache& k = cache(c);
  bool constant = allow_cache && c.is_constant(x.p);
  const int64_t rows = x.rows, cols = x.cols;
  UCC_REQUIRE(rows < INT32_MAX && cols < INT32_MAX, UCC_BAD_ARGS, "sliced GEMM: operand too large");
  const Key key = make_key(x, pad_rows, kSlices);
  if (constant) {
    auto it = k.sliced.find(key);
    if (it != k.sliced.end()) return slice_map(it->second.get(), box_rows);
    S = kSlices;
  }
  auto s = std::make_unique<Sliced>();
  s->rows = rows;
  s->rows_p = (rows + pad_rows - 1) / pad_rows * pad_rows;
  s->kp = (cols + BK - 1) / BK * BK;
  s->S = S;
  const size_t nel = (size_t)S * s->rows_p * s->kp;
  size_t free_b = 0, total_b = 0;
  UCC_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double need = 2.0 * nel + 4.0 * rows;
  // a cached copy keeps a tenth of the memory free for the solver; a temporary 2 GB
  if (constant && need > (double)free_b - 0.1 * (double)total_b) constant = false;
  if (!constant && need > (double)free_b - 2e9) return nullptr;
  if (constant) {
    UCC_CUDA(cudaMalloc(&s->d, sizeof(__nv_bfloat16) * nel));
    UCC_CUDA(cudaMalloc(&s->e, sizeof(int) * rows));
  } else {
    s->tmp = std::make_unique<Scratch>(c, sizeof(__nv_bfloat16) * nel + sizeof(int) * rows + 16);
    s->d = static_cast<__nv_bfloat16*>(s->tmp->p);
    s->e = reinterpret_cast<int*>(static_cast<char*>(s->tmp->p) + ((sizeof(__nv_bfloat16) * nel + 15) / 16) * 16);
  }
  Scratch amax(c, sizeof(unsigned long long) * rows);
  UCC_CUDA(cudaMemsetAsync(amax.p, 0, sizeof(unsigned long long) * rows, c.stream));
  // K chunks of >= 1024 elements, enough blocks to cover the SMs a few times
  const int64_t rblocks = (rows + 31) / 32;
  const int64_t want = std::max<int64_t>(1, (int64_t)k.sms * 8 / rblocks);
  const int64_t kchunk = std::max<int64_t>(1024, (cols + want - 1) / want);
  const dim3 blk(32, 8);
  slice_absmax_kernel<<<dim3((unsigned)((cols + kchunk - 1) / kchunk), (unsigned)rblocks), blk, 0, c.stream>>>(
      x, kchunk, static_cast<unsigned long long*>(amax.p));
  count_kernel_launch();
  slice_digits_kernel<<<dim3((unsigned)(s->kp / 64), (unsigned)(s->rows_p / 32)), blk, 0, c.stream>>>(
      x, s->rows_p, s->kp, static_cast<const unsigned long long*>(amax.p), S, s->d, s->e, k.range);
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
  slice_map(s.get(), box_rows);
  Sliced* raw = s.get();
  if (constant)
    k.sliced[key] = std::move(s);
  else
    temp = std::move(s);
  return raw;
}

}  // namespace tc

// the smallest GEMM the sliced FP64 GEMM takes
constexpr double kSlicedMinWork = 3e7;

static bool sliced_gemm_part(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A,
                             const MatView& B, double beta, double* C, const GemmEpilogue& epi, int S, bool allow_cache,
                             bool& wrote);

// A: M x K, B: N x K (rows = the output's columns)
bool sliced_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B,
                     double beta, double* C, const GemmEpilogue& epi, int S) {
  bool wrote = false;
  const bool ok = sliced_gemm_part(c, M, N, K, alpha, A, B, beta, C, epi, S, true, wrote);
  // a false return lets the caller redo the whole product in FP64, so no chunk may have been
  // written by then
  UCC_REQUIRE(ok || !wrote, UCC_BAD_ARGS, "sliced GEMM: operand outside the sliced range after partial output");
  return ok;
}

bool sliced_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                     const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi,
                     int S) {
  return sliced_gemm_run(c, M, N, K, alpha, MatView::strided(A, M, K, sAm, sAk), MatView::strided(B, N, K, sBn, sBk),
                         beta, C, epi, S);
}

// one sliced product, or the longer of M and N (else K) in halves when the slices exceed one
// launch's limits or the free memory (chunks are sliced as temporaries; a chunk boundary must
// not split a two-stride run)
static bool sliced_gemm_part(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A,
                             const MatView& B, double beta, double* C, const GemmEpilogue& epi, int S, bool allow_cache,
                             bool& wrote) {
  using namespace tc;
  UCC_REQUIRE(S >= 2 && SB * S <= 56, UCC_BAD_ARGS, "sliced GEMM: 2 to 9 slices");
  const double aa = std::fabs(alpha);
  if (!(aa >= 0x1p-20 && aa <= 0x1p20) || M > INT32_MAX || N > INT32_MAX) return false;
  // N tile (pick_bn): no more tiles than 256-column ones would need, padded to multiples of 32
  const int bn = pick_bn(N);
  Cache& k = cache(c);
  {
    const int64_t Mp = (M + BM - 1) / BM * BM, Np = (N + bn - 1) / bn * bn, kp = (K + BK - 1) / BK * BK;
    auto cached = [&](const MatView& x, int box) {
      return allow_cache && k.sliced.count(make_key(x, box, kSlices)) != 0;
    };
    const double needA = cached(A, BM) ? 0.0 : 2.0 * S * (double)Mp * kp;
    const double needB = cached(B, bn) ? 0.0 : 2.0 * S * (double)Np * kp;
    size_t free_b = 0, total_b = 0;
    UCC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const bool too_big = (double)S * Mp >= 2e9 || (double)S * Np >= 2e9 || Np / 32 > 65535 || Mp / 32 > 65535 ||
                         needA + needB > (double)free_b - 4e9;
    if (too_big) {
      MatView x1, x2, y1, y2;
      if (needB >= needA && N > bn) {
        const int64_t n1 = ((N + 1) / 2 + bn - 1) / bn * bn;
        if (B.sub_rows(0, n1, x1) && B.sub_rows(n1, N - n1, x2))
          return sliced_gemm_part(c, M, n1, K, alpha, A, x1, beta, C, epi, S, false, wrote) &&
                 sliced_gemm_part(c, M, N - n1, K, alpha, A, x2, beta, C + n1 * epi.s_n, epi, S, false, wrote);
      }
      const int64_t unit = epi.msplit ? (int64_t)BM * epi.msplit : BM;  // row chunks keep the row split whole
      if (M > unit && needA >= needB) {
        const int64_t m1 = ((M + 1) / 2 + unit - 1) / unit * unit;
        if (m1 < M && A.sub_rows(0, m1, x1) && A.sub_rows(m1, M - m1, x2)) {
          const int64_t off = epi.msplit ? (m1 / epi.msplit) * epi.s_mhi : m1 * epi.s_mhi;
          return sliced_gemm_part(c, m1, N, K, alpha, x1, B, beta, C, epi, S, false, wrote) &&
                 sliced_gemm_part(c, M - m1, N, K, alpha, x2, B, beta, C + off, epi, S, false, wrote);
        }
      }
      // both operands short and K long (or little memory left): K in halves, the second
      // accumulating onto the first
      if (K >= 2 * 4096) {
        const int64_t k1 = ((K + 1) / 2 + BK - 1) / BK * BK;
        if (A.sub_cols(0, k1, x1) && A.sub_cols(k1, K - k1, x2) && B.sub_cols(0, k1, y1) &&
            B.sub_cols(k1, K - k1, y2))
          return sliced_gemm_part(c, M, N, k1, alpha, x1, y1, beta, C, epi, S, false, wrote) &&
                 sliced_gemm_part(c, M, N, K - k1, alpha, x2, y2, 1.0, C, epi, S, false, wrote);
      }
      return false;
    }
  }
  cudaEvent_t ev0 = c.take_event(), ev1 = c.take_event();
  UCC_CUDA(cudaEventRecord(ev0, c.stream));  // the time includes the slicing of non-cached operands
  std::unique_ptr<Sliced> ta, tb;
  // neighbouring M tiles pair up in clusters that share each B slice tile (boxes of bn / 2)
  const int cm = cluster_m((int)((M + BM - 1) / BM));
  Sliced* a = slice_prepare(c, A, BM, BM, S, ta, allow_cache);
  const CUtensorMap amap = a ? a->map : CUtensorMap{};  // copied: A and B may be one cached operand
  Sliced* b = a ? slice_prepare(c, B, bn, bn / cm, S, tb, allow_cache) : nullptr;
  if (!a || !b) {
    c.event_pool.push_back(ev0);
    c.event_pool.push_back(ev1);
    return false;
  }
  const CUtensorMap bmap = b->map;
  wrote = true;
  if (!k.sattr_set) {
    UCC_CUDA(cudaFuncSetAttribute(sliced_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)SLICED_SMEM_BYTES));
    UCC_CUDA(cudaFuncSetAttribute(sliced_gemm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)SLICED_SMEM_BYTES));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * k.sms);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = SLICED_SMEM_BYTES;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    UCC_CUDA(cudaOccupancyMaxActiveClusters(&n, sliced_gemm_kernel<2>, &cfg));
    k.max_pairs_sliced = std::max(1, n);
    k.sattr_set = true;
  }
  SParams p;
  p.M = (int)M;
  p.N = (int)N;
  p.bn = bn;
  p.kblocks = (int)(a->kp / BK);
  p.mtiles = (int)((M + BM - 1) / BM);
  p.ntiles = (int)((N + bn - 1) / bn);
  p.S = S;
  p.gex = std::max(1, S - 2);
  p.a_rows = (int)a->rows_p;
  p.b_rows = (int)b->rows_p;
  p.alpha = alpha;
  p.beta = beta;
  p.C = C;
  p.epi = epi;
  p.ea = a->e;
  p.eb = b->e;
  p.err = k.err;
  p.ksplit = 1;
  p.kchunk = p.kblocks;
  const int tiles = p.mtiles * p.ntiles;
  std::unique_ptr<Scratch> part;
  // split K when the tiles fill the SMs poorly: the split z (chunks of >= 8 K blocks, FP64
  // partials of at most 2 GB) with the shortest time in waves, ceil(tiles z / SMs) / z,
  // a larger z only for a 5 % gain; fixed-order FP64 reduce
  int ks = 1;
  {
    const int zmax = (int)std::min<int64_t>(std::min<int64_t>(p.kblocks / 8, 256),
                                            std::max<int64_t>(1, 8LL * k.sms / tiles));
    double best = (double)((tiles + k.sms - 1) / k.sms);
    for (int z = 2; z <= zmax && 8.0 * M * N * z <= 2e9; z++) {
      const double t = (double)((tiles * z + k.sms - 1) / k.sms) / z;
      if (t < 0.95 * best) {
        best = t;
        ks = z;
      }
    }
  }
  {
    if (ks > 1) {
      p.kchunk = (p.kblocks + ks - 1) / ks;
      p.ksplit = (p.kblocks + p.kchunk - 1) / p.kchunk;
      part = std::make_unique<Scratch>(c, sizeof(double) * M * N * p.ksplit);
      p.C = part->d();
      p.alpha = 1.0;
      p.beta = 0.0;
      p.epi.msplit = 0;
      p.epi.s_mhi = N;
      p.epi.s_n = 1;
    }
  }
  if (cm == 1) {
    sliced_gemm_kernel<1><<<std::min(tiles * p.ksplit, k.sms), THREADS, SLICED_SMEM_BYTES, c.stream>>>(amap, bmap,
                                                                                                        p);
  } else {
    const int groups = (p.mtiles + 1) / 2 * p.ntiles * p.ksplit;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * std::min(groups, k.max_pairs_sliced));
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = SLICED_SMEM_BYTES;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    UCC_CUDA(cudaLaunchKernelEx(&cfg, sliced_gemm_kernel<2>, amap, bmap, p));
  }
  count_kernel_launch();
  c.stats.sliced_gemm_launches++;
  UCC_CUDA(cudaGetLastError());
  if (part) splitk_reduce(c, M, N, p.ksplit, part->d(), alpha, beta, C, epi);
  UCC_CUDA(cudaEventRecord(ev1, c.stream));
  // no synchronisation: temporaries are freed in stream order, the time is resolved with the
  // other GEMM timers and the status flags are read at the next synchronisation (tc_check)
  c.gemm_timers.push_back({ev0, ev1, 2.0 * (double)M * (double)N * (double)K, 2, 0.5 * S * (S + 1)});
  if (c.gemm_timers.size() >= 4096) c.resolve_timers();
  UCC_CUDA(cudaMemcpyAsync(k.pinned, k.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  return true;
}

namespace tc {
// ring layout of a two-part launch: fused stages (A_hi | A_lo | B_hi | B_lo), as many as fit
static void set_fused(Params& p, bool fused) {
  p.fused = fused ? 1 : 0;
  p.stage_bytes = 2 * A_BYTES + 2 * p.bn * BK * 2;
  p.nst = fused ? (int)std::min<size_t>(STAGES, GEMM_RING / (size_t)p.stage_bytes) : STAGES;
}

static void set_gemm_attrs(Cache& k) {
  if (k.attr_set) return;
  UCC_CUDA(cudaFuncSetAttribute(gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM_BYTES));
  UCC_CUDA(cudaFuncSetAttribute(gemm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM_BYTES));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * k.sms);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = GEMM_SMEM_BYTES;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  UCC_CUDA(cudaOccupancyMaxActiveClusters(&n, gemm_kernel<2>, &cfg));
  k.max_pairs = std::max(1, n);
  k.attr_set = true;
}

// one persistent launch over `work` tiles (output tiles x problems or K chunks): one CTA
// per SM, or pairs of CTAs in clusters when cm = 2
static void launch_gemm(Ctx& c, Cache& k, int cm, int work, const CUtensorMap& ahi, const CUtensorMap& alo,
                        const CUtensorMap& bhi, const CUtensorMap& blo, const CUtensorMap& a2hi,
                        const CUtensorMap& a2lo, const CUtensorMap& amid, const CUtensorMap& bmid, const Params& p) {
  set_gemm_attrs(k);
  if (cm == 1) {
    gemm_kernel<1><<<std::min(work, k.sms), THREADS, GEMM_SMEM_BYTES, c.stream>>>(ahi, alo, bhi, blo, a2hi, a2lo,
                                                                                  amid, bmid, p);
  } else {
    const int groups = (p.mtiles + 1) / 2 * p.ntiles * (p.nprob ? p.nprob : (p.ksplit > 1 ? p.ksplit : 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * std::min(groups, k.max_pairs));
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = GEMM_SMEM_BYTES;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    UCC_CUDA(cudaLaunchKernelEx(&cfg, gemm_kernel<2>, ahi, alo, bhi, blo, a2hi, a2lo, amid, bmid, p));
  }
  count_kernel_launch();
  c.stats.tc_gemm_launches++;
  UCC_CUDA(cudaGetLastError());
}
}  // namespace tc

// A: M x K, B: N x K (rows = the output's columns)
void tc_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B,
                 double beta, double* C, const GemmEpilogue& epi, int parts, int kc) {
  using namespace tc;
  UCC_REQUIRE(parts == 2 || parts == 3, UCC_BAD_ARGS, "tensor-core GEMM: 2 or 3 split parts");
  Cache& k = cache(c);
  std::unique_ptr<Split> ta, tb;
  const int bn = pick_bn(N);
  const int cm = cluster_m((int)((M + BM - 1) / BM));
  // the maps are copied at once: A and B may be one cached operand read with two boxes
  Split* a = prepare(c, A, BM, ta, parts);
  const CUtensorMap a_hi = a->mhi, a_lo = a->mlo, a_mid = a->mmid;
  Split* b = prepare(c, B, bn / cm, tb, parts);
  const CUtensorMap b_hi = b->mhi, b_lo = b->mlo, b_mid = b->mmid;
  Params p;
  p.M = (int)M;
  p.N = (int)N;
  p.kblocks = (int)(a->kp / BK);
  p.mtiles = (int)((M + BM - 1) / BM);
  p.bn = bn;
  p.ntiles = (int)((N + bn - 1) / bn);
  p.alpha = alpha;
  p.beta = beta;
  p.C = C;
  p.epi = epi;
  p.err = k.err;
  p.nprob = 0;
  p.a_row0 = p.b_row0 = nullptr;
  p.c_off = nullptr;
  p.ksplit = 1;
  p.kchunk = p.kblocks;
  const int tiles = p.mtiles * p.ntiles;
  // tiles that fill the SMs poorly and a long K: split K (chunks of >= 4 K blocks, FP64
  // partials of at most 2 GB) for the shortest time in waves, ceil(tiles z / SMs) / z, a
  // larger z only for a 5 % gain; fixed-order reduce
  std::unique_ptr<Scratch> part;
  p.kc = kc > 0 && kc < p.kblocks ? kc : 0;
  if (p.kc == 0 && p.kblocks >= 8) {
    int ks = 1;
    const int zmax = (int)std::min<int64_t>(std::min<int64_t>(p.kblocks / 4, 256),
                                            std::max<int64_t>(1, 8LL * k.sms / tiles));
    double best = (double)((tiles + k.sms - 1) / k.sms);
    for (int z = 2; z <= zmax && 8.0 * M * N * z <= 2e9; z++) {
      const double t = (double)((tiles * z + k.sms - 1) / k.sms) / z;
      if (t < 0.95 * best) {
        best = t;
        ks = z;
      }
    }
    if (ks > 1) {
      p.kchunk = (p.kblocks + ks - 1) / ks;
      p.ksplit = (p.kblocks + p.kchunk - 1) / p.kchunk;
      part = std::make_unique<Scratch>(c, sizeof(double) * M * N * p.ksplit);
      p.C = part->d();
      p.alpha = 1.0;
      p.beta = 0.0;
      p.epi.msplit = 0;
      p.epi.s_mhi = N;
      p.epi.s_n = 1;
    }
  }
  cudaEvent_t ev0 = c.take_event(), ev1 = c.take_event();
  UCC_CUDA(cudaEventRecord(ev0, c.stream));
  p.nterms = 1;
  p.a_row1 = p.b_row1 = nullptr;
  p.C32 = nullptr;
  p.nparts = parts;
  set_fused(p, parts == 2 && p.kc == 0);
  launch_gemm(c, k, cm, tiles * p.ksplit, a_hi, a_lo, b_hi, b_lo, a_hi, a_lo, parts == 3 ? a_mid : a_hi,
              parts == 3 ? b_mid : b_hi, p);
  if (part) splitk_reduce(c, M, N, p.ksplit, part->d(), alpha, beta, C, epi);
  UCC_CUDA(cudaEventRecord(ev1, c.stream));
  // no synchronisation (see sliced_gemm_part)
  c.gemm_timers.push_back({ev0, ev1, 2.0 * (double)M * (double)N * (double)K, 1});
  if (c.gemm_timers.size() >= 4096) c.resolve_timers();
  UCC_CUDA(cudaMemcpyAsync(k.pinned, k.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
}

// the status of the tensor-core launches since the last check, after a synchronisation of
// the stream: a pipeline wait that timed out, or a sliced operand whose row maximum is
// beyond 2^498 (the product of such rows is not formed; FP64 covers them)
void tc_check(Ctx& c) {
  if (!c.tc_cache) return;
  tc::Cache& k = *static_cast<tc::Cache*>(c.tc_cache.get());
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  const int herr = k.pinned[0], hrange = k.pinned[1];
  if (!herr && !hrange) return;
  k.pinned[0] = k.pinned[1] = 0;
  UCC_CUDA(cudaMemsetAsync(k.err, 0, 2 * sizeof(int), c.stream));
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  if (herr) throw Error(UCC_DEVICE_TIMEOUT, "tensor-core GEMM: a pipeline wait timed out");
  throw Error(UCC_BAD_ARGS, "sliced FP64 GEMM: an operand row maximum is beyond 2^498; use PRECISION FP64");
}

// a device-side wait of limit_ns that nothing completes: the kernel returns once it runs
// out and the status check that follows every tensor-core launch reports
// UCC_DEVICE_TIMEOUT; the stream and the context stay usable
void wait_selftest(Ctx& c, unsigned long long limit_ns) {
  tc::Cache& k = tc::cache(c);
  tc::wait_selftest_kernel<<<1, 32, 0, c.stream>>>(k.err, limit_ns);
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
  UCC_CUDA(cudaMemcpyAsync(k.pinned, k.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  tc_check(c);
}

void tc_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi, int parts,
                 int kc) {
  tc_gemm_run(c, M, N, K, alpha, MatView::strided(A, M, K, sAm, sAk), MatView::strided(B, N, K, sBn, sBk), beta, C,
              epi, parts, kc);
}

void tc_gemm_run(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi) {
  tc_gemm_run(c, M, N, K, alpha, A, sAm, sAk, B, sBk, sBn, beta, C, epi, 2, 0);
}

bool tc_eligible(int64_t M, int64_t N, int64_t K) {
  // small problems stay on the FP64 path; the tensor tile is 128 x 256 x 64.  A small
  // output with a long K (a reduction such as Fmi, 32 x 32 x 3.3e6 at no=32/nv=320:
  // 6.7 GFLOP, ~6 ms on the FP64 pipe) runs split-K over the SMs despite its mostly empty tile
  const bool reduction = K >= 65536 && (double)M * N * K >= 1e9;
  if ((std::max(M, N) < 64 && !reduction) || K < 16 || (double)M * N * K < 1e7) return false;
  return M <= INT32_MAX && N <= INT32_MAX;
}

// C (strides sCm, sCn) = alpha A B + beta C with A: M x K and B: N x K views; a short M becomes
// the narrow N tile of C^T = B^T A^T so that the long side fills the 128-row MMA tile
void tc_gemm_oriented(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B,
                      double beta, double* C, int64_t sCm, int64_t sCn, int parts, int kc) {
  GemmEpilogue epi;
  epi.msplit = 0;
  if (M <= 256 && N > M) {
    epi.s_mhi = sCn;
    epi.s_n = sCm;
    tc_gemm_run(c, N, M, K, alpha, B, A, beta, C, epi, parts, kc);
  } else {
    epi.s_mhi = sCm;
    epi.s_n = sCn;
    tc_gemm_run(c, M, N, K, alpha, A, B, beta, C, epi, parts, kc);
  }
}

void tc_gemm_oriented(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm,
                      int64_t sAk, const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm,
                      int64_t sCn, int parts, int kc) {
  tc_gemm_oriented(c, M, N, K, alpha, MatView::strided(A, M, K, sAm, sAk), MatView::strided(B, N, K, sBn, sBk), beta,
                   C, sCm, sCn, parts, kc);
}

// FP64-accurate GEMM on the tensor cores (sliced operands) for the FP64 work of the MIXED
// form; false when the problem is too small for it or outside its exponent range
bool sliced_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B,
                 double beta, double* C, int64_t sCm, int64_t sCn) {
  // a short K (a few occupied indices) leaves too little work per slice and output: routing
  // the K = 16 contractions of a no=16/nv=160 CCSD solve here instead of the DFMA kernel
  // (operands sliced per call, 45 padded products, the 9-order epilogue) made its sweeps
  // slower (203 -> 220 ms per solve), and the K = 32 ones of no=32/nv=320 (outputs of 1e8,
  // 6.7 GFLOP) made its record sweeps slower too (606 -> 625 ms at 6 digits, 877 -> 946 ms
  // at 8): the per-order epilogue passes over the output cost more than the DFMA work
  if (K < 48 || (double)M * N * K < kSlicedMinWork || M > INT32_MAX || N > INT32_MAX) return false;
  // the output must fill at least 1/16 of its 128 x (N rounded to 32) tiles
  const int64_t lo = std::min(M, N), hi = std::max(M, N);
  if (16.0 * (double)lo * hi < (double)((hi + 127) / 128 * 128) * (double)((lo + 31) / 32 * 32)) return false;
  GemmEpilogue epi;
  epi.msplit = 0;
  // a record sweep's products carry the digits its anchor needs; everything else all of them
  const int digits = c.anchors.mode == 1 ? std::min(tc::kSlices, std::max(2, c.anchors.digits)) : tc::kSlices;
  if (M <= 256 && N > M) {  // the short side becomes the (narrow) N tile
    epi.s_mhi = sCn;
    epi.s_n = sCm;
    return sliced_gemm_run(c, N, M, K, alpha, B, A, beta, C, epi, digits);
  }
  epi.s_mhi = sCm;
  epi.s_n = sCn;
  return sliced_gemm_run(c, M, N, K, alpha, A, B, beta, C, epi, digits);
}

bool sliced_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm, int64_t sCn) {
  return sliced_gemm(c, M, N, K, alpha, MatView::strided(A, M, K, sAm, sAk), MatView::strided(B, N, K, sBn, sBk), beta,
                     C, sCm, sCn);
}

bool mixed_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B, double beta,
                double* C, int64_t sCm, int64_t sCn) {
  if (!tc_eligible(M, N, K)) return false;
  tc_gemm_oriented(c, M, N, K, alpha, A, B, beta, C, sCm, sCn, 2, 0);
  return true;
}

bool mixed_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm, int64_t sCn) {
  return mixed_gemm(c, M, N, K, alpha, MatView::strided(A, M, K, sAm, sAk), MatView::strided(B, N, K, sBn, sBk), beta,
                    C, sCm, sCn);
}

// ------------------------------------------------------------------------------------
// (T) on the tensor cores: A_x^T = [<xe|ab> ; -t2[x][m][a][b]] stacked over x as
// [no*nv^2][K'] and B_yz^T = [t2[y][z][c][e] ; <zy|mc>] stacked over (y,z) as [no^2*nv][K']
// (K' = nv + no padded to 64), split once per (T) call; each of the six terms of a tuple
// batch is one batched launch whose problems are the tuples of the batch.
// ------------------------------------------------------------------------------------
namespace tc {
// dst[(row0 + r) * ld + col0 + k] (hi/lo) = scale * src[(r / rsplit) * sr_hi + (r % rsplit) * sr + k*sk],
// r < rows, k < cols; 32x32 tiles through shared memory so that the destination rows are
// written coalesced
__global__ void split_into_kernel(int64_t rows, int64_t cols, const double* src, int64_t rsplit, int64_t sr_hi,
                                  int64_t sr, int64_t sk, double scale, __nv_bfloat16* hi, __nv_bfloat16* lo,
                                  int64_t ld, int64_t row0, int64_t col0) {
  __shared__ double t[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int64_t r = r0 + threadIdx.x, k = k0 + yy;
    const double x = (r < rows && k < cols) ? src[(r / rsplit) * sr_hi + (r % rsplit) * sr + k * sk] : 0.0;
    t[yy][threadIdx.x] = scale == 1.0 ? x : scale * x;
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int64_t r = r0 + yy, k = k0 + threadIdx.x;
    if (r < rows && k < cols) {
      // in FP32 from the truncated value (2^-23, below the lo part's 2^-17): no FP64 pipe work
      const float f = f64_to_f32_trunc(t[threadIdx.x][yy]);
      const __nv_bfloat16 h = __float2bfloat16_rn(f);
      const int64_t o = (row0 + r) * ld + col0 + k;
      hi[o] = h;
      lo[o] = __float2bfloat16_rn(f - __bfloat162float(h));
    }
  }
}

struct Triples {
  Split A, A2, B;  // A2: A with its (a,b) row pairs in (b,a) order
  int bn = BN;     // N tile over the virtual index c (pick_bn)
  int* d_arow = nullptr;
  int* d_brow = nullptr;
  int64_t* d_coff = nullptr;
  ~Triples() {
    if (d_arow) cudaFree(d_arow);
    if (d_brow) cudaFree(d_brow);
    if (d_coff) cudaFree(d_coff);
  }
};

static void split_into(Ctx& c, int64_t rows, int64_t cols, const double* src, int64_t sr, int64_t sk, double scale,
                       Split& dst, int64_t row0, int64_t col0, int64_t rsplit = 0, int64_t sr_hi = 0) {
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  UCC_REQUIRE(grid.y <= 65535, UCC_BAD_ARGS, "split_into: too many rows");
  if (rsplit <= 0) rsplit = rows;  // one level: r * sr
  split_into_kernel<<<grid, dim3(32, 8), 0, c.stream>>>(rows, cols, src, rsplit, sr_hi, sr, sk, scale, dst.hi, dst.lo,
                                                        dst.kp, row0, col0);
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
}

static void alloc_split(Split& s, int64_t rows, int64_t kp, cudaStream_t st) {
  s.rows = rows;
  s.kp = kp;
  UCC_CUDA(cudaMalloc(&s.hi, sizeof(__nv_bfloat16) * rows * kp));
  UCC_CUDA(cudaMalloc(&s.lo, sizeof(__nv_bfloat16) * rows * kp));
  UCC_CUDA(cudaMemsetAsync(s.hi, 0, sizeof(__nv_bfloat16) * rows * kp, st));
  UCC_CUDA(cudaMemsetAsync(s.lo, 0, sizeof(__nv_bfloat16) * rows * kp, st));
}
}  // namespace tc

bool mixed_triples_prepare(Ctx& c, int max_batch) {
  using namespace tc;
  const int64_t no = c.no, nv = c.nv, nv2 = nv * nv, kp = (nv + no + BK - 1) / BK * BK;
  if (nv < 64) return false;  // small virtual spaces stay on the FP64 path
  Cache& k = cache(c);
  auto T = std::make_shared<Triples>();
  alloc_split(T->A, no * nv2, kp, c.stream);
  alloc_split(T->A2, no * nv2, kp, c.stream);
  alloc_split(T->B, no * no * nv, kp, c.stream);
  const double* t2 = c.get("T").p + no * nv;
  const double* Vovvv = c.get("Vovvv").p;
  const double* Vooov = c.get("Vooov").p;
  for (int64_t x = 0; x < no; x++) {
    split_into(c, nv2, nv, Vovvv + x * nv * nv2, 1, nv2, 1.0, T->A, x * nv2, 0);   // <xe|ab>
    split_into(c, nv2, no, t2 + x * no * nv2, 1, nv2, -1.0, T->A, x * nv2, nv);   // -t2[x][m][a][b]
    // the same rows in (b,a) order: row b*nv + a
    split_into(c, nv2, nv, Vovvv + x * nv * nv2, nv, nv2, 1.0, T->A2, x * nv2, 0, nv, 1);
    split_into(c, nv2, no, t2 + x * no * nv2, nv, nv2, -1.0, T->A2, x * nv2, nv, nv, 1);
  }
  split_into(c, no * no * nv, nv, t2, nv, 1, 1.0, T->B, 0, 0);  // t2[y][z][c][e]
  for (int64_t y = 0; y < no; y++)
    for (int64_t z = 0; z < no; z++)  // <zy|mc>
      split_into(c, nv, no, Vooov + (z * no + y) * no * nv, 1, nv, 1.0, T->B, (y * no + z) * nv, nv);
  make_map(&T->A.mhi, T->A.hi, T->A.rows, kp, BM);
  make_map(&T->A.mlo, T->A.lo, T->A.rows, kp, BM);
  make_map(&T->A2.mhi, T->A2.hi, T->A2.rows, kp, BM);
  make_map(&T->A2.mlo, T->A2.lo, T->A2.rows, kp, BM);
  T->bn = pick_bn(nv);
  // M = nv^2 rows per tuple: always two or more M tiles, so the launches pair CTAs that
  // share the B tile (boxes of bn / 2 rows)
  make_map(&T->B.mhi, T->B.hi, T->B.rows, kp, T->bn / 2);
  make_map(&T->B.mlo, T->B.lo, T->B.rows, kp, T->bn / 2);
  UCC_CUDA(cudaMalloc(&T->d_arow, sizeof(int) * 6 * max_batch));  // 3 term pairs x 2 terms
  UCC_CUDA(cudaMalloc(&T->d_brow, sizeof(int) * 6 * max_batch));
  UCC_CUDA(cudaMalloc(&T->d_coff, sizeof(int64_t) * 3 * max_batch));
  k.triples = T;
  set_gemm_attrs(k);
  return true;
}

void mixed_triples_release(Ctx& c) {
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  tc::cache(c).triples.reset();
}

// W3 of nb tuples as three FP32 partial arrays, one per pair of terms: pair pq writes
// W3 + (pq * nb + b) * S for tuple b with beta 0 (no read-modify-write of W3 in the
// epilogue), S = nv^3 in the plain [a][b][c] layout (tblk = 0) or tblk^3 * 512 in the
// blocked layout of w3_block_offset; triples_energy_f32 adds the three while staging its
// tiles.  The three launches go out back to back with their own row tables; the caller
// synchronises.
bool mixed_triples_batch(Ctx& c, int nb, const int* tuples, float* W3, int tblk) {
  using namespace tc;
  Cache& k = cache(c);
  Triples& T = *k.triples;
  const int64_t no = c.no, nv = c.nv, nv2 = nv * nv, nv3 = nv2 * nv;
  const int64_t per = tblk ? (int64_t)tblk * tblk * tblk * 512 : nv3;  // floats per tuple and partial
  UCC_REQUIRE(!tblk || (tblk >= (nv + 7) / 8 && per < ((int64_t)1 << 31)), UCC_BAD_ARGS,
              "mixed (T): blocked W3 needs whole 8-wide blocks and < 2^31 floats per tuple");
  TriplesTerm terms[6];
  triples_terms(nv, terms);
  // The six terms in pairs that write the same W3 layout: the first term of a pair uses
  // A's natural (a,b) rows, the second the (b,a) copy, so that one tile accumulates both
  // in tensor memory; every pair's fastest-varying output row index has W3 stride 1 or
  // its column index does.
  const int pairs[3][2] = {{0, 5}, {1, 2}, {4, 3}};
  std::vector<int> arow(6 * nb), brow(6 * nb);
  std::vector<int64_t> coff(3 * nb);
  for (int pq = 0; pq < 3; pq++) {
    for (int b = 0; b < nb; b++) coff[pq * nb + b] = ((int64_t)pq * nb + b) * per;
    for (int t = 0; t < 2; t++) {
      const TriplesTerm& tm = terms[pairs[pq][t]];
      for (int b = 0; b < nb; b++) {
        const int* ijk = tuples + 3 * b;
        arow[(2 * pq + t) * nb + b] = (int)(ijk[tm.x] * nv2);
        brow[(2 * pq + t) * nb + b] = (int)((ijk[tm.y] * no + ijk[tm.z]) * nv);
      }
    }
  }
  UCC_CUDA(cudaMemcpyAsync(T.d_coff, coff.data(), sizeof(int64_t) * 3 * nb, cudaMemcpyHostToDevice, c.stream));
  UCC_CUDA(cudaMemcpyAsync(T.d_arow, arow.data(), sizeof(int) * 6 * nb, cudaMemcpyHostToDevice, c.stream));
  UCC_CUDA(cudaMemcpyAsync(T.d_brow, brow.data(), sizeof(int) * 6 * nb, cudaMemcpyHostToDevice, c.stream));
  cudaEvent_t ev0 = c.take_event(), ev1 = c.take_event();
  UCC_CUDA(cudaEventRecord(ev0, c.stream));
  for (int pq = 0; pq < 3; pq++) {
    const TriplesTerm& t0 = terms[pairs[pq][0]];
    Params p;
    p.M = (int)nv2;
    p.N = (int)nv;
    p.kblocks = (int)(T.A.kp / BK);
    p.mtiles = (int)((nv2 + BM - 1) / BM);
    p.bn = T.bn;
    p.ntiles = (int)((nv + T.bn - 1) / T.bn);
    p.alpha = 1.0;
    p.beta = 0.0;
    p.C = nullptr;
    p.C32 = W3;  // W3 in FP32: its rounding (~6e-8) is far below the split products' (~5e-6)
    p.tblk = tblk;
    p.epi.msplit = nv;
    p.epi.s_mhi = t0.su;
    p.epi.s_mlo = t0.sv;
    p.epi.s_n = t0.sw;
    p.err = k.err;
    p.nprob = nb;
    p.ksplit = 1;
    p.kchunk = p.kblocks;
    p.a_row0 = T.d_arow + 2 * pq * nb;
    p.b_row0 = T.d_brow + 2 * pq * nb;
    p.c_off = T.d_coff + pq * nb;
    p.nterms = 2;
    p.a_row1 = T.d_arow + (2 * pq + 1) * nb;
    p.b_row1 = T.d_brow + (2 * pq + 1) * nb;
    const int tiles = p.mtiles * p.ntiles * nb;
    p.nparts = 2;
    p.kc = 0;
    set_fused(p, true);
    launch_gemm(c, k, 2, tiles, T.A.mhi, T.A.mlo, T.B.mhi, T.B.mlo, T.A2.mhi, T.A2.mlo, T.A.mhi, T.B.mhi, p);
  }
  UCC_CUDA(cudaEventRecord(ev1, c.stream));
  // timed with the other GEMMs (resolved lazily); the status flags are read at the next check
  c.gemm_timers.push_back({ev0, ev1, 2.0 * 6.0 * (double)nv2 * (double)nv * (double)(nv + no) * nb, 1});
  if (c.gemm_timers.size() >= 4096) c.resolve_timers();
  UCC_CUDA(cudaMemcpyAsync(k.pinned, k.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  return true;
}

}  // namespace ucc
