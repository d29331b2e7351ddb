// Tensor-core (tcgen05) Legendre sandwich of one modified-Euler step at
// truncation M = 106 (160 x 320 Gauss grid), FP32 fast path, 3xTF32, and its
// adjoint.
//
// The arithmetic is that of k_spectral_tc / k_spectral_adj_tc (tc_legendre.cu);
// only the tiling differs.  At J = 160 one CTA's operands for the one-shot GEMMs
// of the smaller truncations would take 320 KB (A1: 128 rows x 160 latitudes,
// hi + lo, per parity; B1 the same size), beyond the 227 KB a CTA may hold.  So:
//   GEMM1 (forward Legendre; the adjoint's transposed inverse Legendre) runs
//   over 5 chunks of 16 latitude pairs.  For each chunk the inputs of its 8
//   members x 16 j' are read straight from global memory (the two mirror
//   latitudes of a pair are lanes l and l ^ 16 of a warp, which exchange their
//   values by shuffles), split into hi / lo TF32 and written as the K-slice
//   [P at j' | H at j'] of both parities' A operands, while the basis slice of
//   the chunk arrives by bulk copy.  Two stages: the MMAs of one chunk run while
//   the next chunk is formed.  D1 accumulates in TMEM over the chunks.
//   GEMM2 (inverse Legendre; the adjoint's transposed forward Legendre) runs per
//   parity over two halves of the 160 output columns [P at j' | H at j'], with
//   the basis halves double-buffered.
// Every wait is bounded; on a timeout the CTA sets the device error word, waits
// (bounded) for what it issued, frees its TMEM and returns.
#include "swp_internal.h"
#include "spec_common.cuh"
#include "tc_common.cuh"

namespace swp {

namespace {
struct T106 {
  static constexpr int M = 106, J = 160, JH = 80, MT = 8, CNT = 107, ROWS = 128;
  static constexpr int N1 = 64;                          // >= ceil(107 / 2), multiple of 16
  static constexpr int K2 = 56;                          // >= ceil(107 / 2), multiple of 8
  static constexpr int N2 = 2 * JH;                      // 160 output columns
  static constexpr int N2H = N2 / 2;                     // 80: one GEMM2 column half
  static constexpr int CJ = 16, NCH = JH / CJ;           // 5 chunks of 16 latitude pairs
  static constexpr int KC = 2 * CJ;                      // K columns of a chunk: P | H
  static constexpr int ACH = 2 * ROWS * KC;              // one parity's A chunk, hi + lo
  static constexpr int BCH = 2 * N1 * KC;                // one parity's B1 chunk, hi + lo
  static constexpr int STAGE = 2 * ACH + 2 * BCH;        // both parities (24576 floats, 96 KB)
  static constexpr int B1 = NCH * 2 * BCH;               // packed B1 floats per m
  static constexpr int B2H = 2 * N2H * K2;               // one parity's B2 column half, hi + lo
  static constexpr int BLOCK = B1 + 4 * B2H;             // packed basis floats per m
  static constexpr int OST = 2 * J + 2;                  // output staging row stride
  static constexpr int COEF = 5 * MT * CNT;
  static constexpr int TMEM_COLS = 512;                  // D1: 2 x 128; D2: 2 x 160 (reusing D1's)
  static constexpr int NWPAIR = (MT * J / 2 + 255) / 256;  // write-out latitude pairs per thread
  // forward, after GEMM1: A2 operands [par][hi, lo] (112 used rows) | D1 staging
  // (GEMM2 buffer 1 once read) | GEMM2 buffer 0
  static constexpr int A2 = 112 * K2;
  static constexpr int RES = 8 * CNT * 16;               // [g][n-m][member, re/im]
  static constexpr int OFF_RES = 4 * A2;
  static constexpr int OFF_BUF0 = OFF_RES + RES;
  static constexpr int REGION = OFF_BUF0 + B2H > 2 * STAGE ? OFF_BUF0 + B2H : 2 * STAGE;
  // adjoint, after GEMM1': A2' operands (128 rows) | D1' staging (buffer 1) | buffer 0
  static constexpr int AA2 = ROWS * K2;
  static constexpr int ARES = 7 * CNT * 16;
  static constexpr int AOFF_RES = 4 * AA2;
  static constexpr int AOFF_BUF0 = AOFF_RES + ARES;
  static constexpr int AREGION = AOFF_BUF0 + B2H > 2 * STAGE ? AOFF_BUF0 + B2H : 2 * STAGE;
  static constexpr int ANOUT = 12;                       // 8 P slots + 4 H slots
  static constexpr int AOFF_GP = ANOUT * MT * OST;       // the Phibar terms [MT][J / 2], after the staging

  static_assert(NCH * CJ == JH && CJ == 16, "chunks of 16 latitude pairs");
  static_assert(B2H <= RES && B2H <= ARES, "buffer 1 reuses the D1 staging");
  static_assert(3 * A2 + ROWS * K2 <= OFF_BUF0, "A2 over-read stays clear of buffer 0");
  static_assert(7 * MT * OST <= OFF_RES, "output staging");
  static_assert(AOFF_GP + MT * JH <= AREGION, "adjoint output staging and Phibar terms");
  static_assert(N1 * KC * 4 == (N1 / 8) * (KC / 4) * 128, "B1 lo tile follows its hi tile");
  static_assert(N2H * K2 * 4 == (N2H / 8) * (K2 / 4) * 128, "B2 lo tile follows its hi tile");
  static_assert((AREGION + COEF) * 4 + 256 <= 227 * 1024, "shared memory");
};
typedef T106 S;

__host__ __device__ constexpr int group_p106(int g) {
  return g == 0 ? SP_PHI1 : g == 1 ? SP_PHI2 : g == 2 ? SP_D1 : g == 3 ? SP_D2 : g == 4 ? SP_E1
       : g == 5 ? SP_IPHI : g == 6 ? SP_ID : SP_IE;
}
__host__ __device__ constexpr int group_h106(int g) {
  return g == 0 ? SH_PHI1 : g == 2 ? SH_D1 : g == 3 ? SH_D2 : g == 4 ? SH_E1 : -1;
}
// the Fourier fields the modified-Euler combination reads (eta, delta, Phi,
// A..G) <-> register slots of the prefetched chunk inputs
__host__ __device__ constexpr int field106(int q) {
  return q == 0 ? F_ETA : q == 1 ? F_DELTA : q == 2 ? F_PHI : F_A + (q - 3);
}
__host__ __device__ constexpr int slot106(int f) {
  return f == F_ETA ? 0 : f == F_DELTA ? 1 : f == F_PHI ? 2 : (f >= F_A && f <= F_G) ? f - F_A + 3 : 0;
}
static_assert(F_G - F_A + 4 == 11, "prefetched fields");
__host__ __device__ constexpr int adj_hslot106(int q) {  // H result of GEMM2' row group q, or -1
  return q == 0 ? 0 : q == 2 ? 1 : q == 3 ? 2 : q == 4 ? 3 : -1;
}

// The MMAs are issued by warp 0 as a whole (warp-collective forms, one elected
// lane issues), with the descriptors of a K-sweep built once and advanced by
// 256 bytes (8 TF32 columns of the core-matrix layout) per K-step.
// the three products of one 3xTF32 K-sweep into d_tmem (operands of K columns)
template <int K>
__device__ __forceinline__ void mma3(uint32_t d_tmem, uint32_t aH, uint32_t aL, uint32_t bH, uint32_t bL,
                                     uint32_t idesc) {
  constexpr uint32_t sbo = (uint32_t)(K / 4) * 128u;
  const uint64_t dAH = tc::make_desc(aH, 128, sbo), dAL = tc::make_desc(aL, 128, sbo);
  const uint64_t dBH = tc::make_desc(bH, 128, sbo), dBL = tc::make_desc(bL, 128, sbo);
#pragma unroll
  for (int kk = 0; kk < K / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBH, off), idesc, kk > 0);
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBL, off), idesc, 1);
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAL, off), tc::desc_advance(dBH, off), idesc, 1);
  }
}
// one chunk of the GEMM1 sweep in two MMAs per K-step (a_hi [b_hi; b_lo], then
// a_lo b_hi onto the second half); the first MMA of the first chunk overwrites
__device__ __forceinline__ void mma2_chunk(uint32_t d_tmem, uint32_t aH, uint32_t aL, uint32_t bH, bool first,
                                           uint32_t idesc_2n, uint32_t idesc_n) {
  constexpr uint32_t sbo = (uint32_t)(S::KC / 4) * 128u;
  const uint64_t dAH = tc::make_desc(aH, 128, sbo), dAL = tc::make_desc(aL, 128, sbo);
  const uint64_t dBH = tc::make_desc(bH, 128, sbo);
#pragma unroll
  for (int kk = 0; kk < S::KC / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBH, off), idesc_2n,
                      (first && kk == 0) ? 0u : 1u);
    tc::mma_tf32_warp(d_tmem + (uint32_t)S::N1, tc::desc_advance(dAL, off), tc::desc_advance(dBH, off), idesc_n, 1);
  }
}

// Warp 0's record of the CTA's mbarriers: the phases it armed on each (a bulk
// copy or an MMA commit) and how many of them it has waited for, so that every
// wait names the next phase and the drain after a timeout waits for exactly the
// phases still open.  Every lane of warp 0 keeps the same record; the copies
// and commits are issued by one elected lane.  Barriers: 0, 1 B1 chunk copies
// per stage; 2, 3 GEMM1 commits per stage; 4, 5 B2 half copies per buffer;
// 6, 7 GEMM2 commits per buffer.
struct BarLog {
  static constexpr int NB = 8;
  uint64_t* bar;
  int iss[NB], wtd[NB];
  __device__ explicit BarLog(uint64_t* b) : bar(b) {
#pragma unroll
    for (int q = 0; q < NB; ++q) iss[q] = wtd[q] = 0;
  }
  __device__ void copy(int q, void* dst, const void* src, uint32_t bytes) {
    tc::bulk_g2s_warp(dst, src, bytes, &bar[q]);
    ++iss[q];
  }
  __device__ void commit(int q) {
    tc::mma_commit_warp(&bar[q]);
    ++iss[q];
  }
  __device__ bool wait(int q, uint32_t limit) {
    if (!tc::mbar_wait_bounded_warp(&bar[q], (uint32_t)(wtd[q] & 1), limit)) return false;
    ++wtd[q];
    return true;
  }
  __device__ void drain() {
    for (int q = 0; q < NB; ++q)
      while (wtd[q] < iss[q])
        if (!wait(q, 1u << 20)) break;
  }
};

constexpr uint32_t B1_BYTES = 2 * S::BCH * sizeof(float), B2_BYTES = S::B2H * sizeof(float);

// CTA set-up shared by both kernels, by warp 0: the mbarriers, the first two
// B1 chunk copies, TMEM.
__device__ __forceinline__ void setup_chunks(BarLog& bl, float* sR, const float* mblock, uint32_t* tslot,
                                             int* sflag) {
  if ((threadIdx.x >> 5) != 0) return;
  if (threadIdx.x == 0) {
    *sflag = 0;
#pragma unroll
    for (int q = 0; q < BarLog::NB; ++q) tc::mbar_init(&bl.bar[q], 1);
    tc::fence_mbar_init();
  }
  __syncwarp();
  for (int s = 0; s < 2; ++s)
    bl.copy(s, sR + (size_t)s * S::STAGE + 2 * S::ACH, mblock + (size_t)s * 2 * S::BCH, B1_BYTES);
  tc::tmem_alloc(tslot, S::TMEM_COLS);
  tc::tmem_relinquish();
}

// The thread's place in a chunk: member bt, latitude pair jl of the chunk, side
// (0: j', 1: its mirror J - 1 - j').  A warp holds 4 members x 4 pairs x 2
// sides, lanes l and l ^ 16 the two latitudes of a pair.  Its A stores then hit
// 32 distinct banks: the bank of an entry is 4 (row % 8) + k % 4 with
// row % 8 = 2 (bt % 4) + component, and the two sides store opposite
// components first.
struct ChunkLane {
  int bt, jl, side;
  __device__ ChunkLane() {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    bt = (warp & 1) * 4 + ((lane >> 2) & 3);
    jl = (warp >> 1) * 4 + (lane & 3);
    side = lane >> 4;
  }
};

// GEMM1 over the latitude chunks into D1 (TMEM columns [128 par, 128 par + 128)).
// fetch(ch, raw) issues the global loads of the thread's inputs at (member,
// j' = 16 ch + jl) into registers -- one chunk ahead, so that their latency
// overlaps the stores and barriers of the current chunk; the caller has fetched
// chunk 0.  form(ch, raw, vp, vh) gives the values of the 8 row groups on the P and
// the H columns, already summed with the mirror latitude: symmetric on side 0,
// antisymmetric on side 1.  Parity 0 takes the symmetric P sums and the
// antisymmetric H sums, parity 1 the reverse, so the side 0 thread writes parity
// 0's P columns and parity 1's H columns, the side 1 thread the other two.
// Returns false (the same value in every thread) when a wait ran out.
template <class Raw, class Fetch, class Form>
__device__ __forceinline__ bool gemm1_chunks(BarLog& bl, float* sR, const float* mblock, uint32_t tbase,
                                             int* sflag, uint32_t lim, const ChunkLane& cl, Raw& raw, Fetch fetch,
                                             Form form) {
  const uint32_t rbase = tc::smem_u32(sR);
  const uint32_t idesc1 = tc::idesc_tf32(S::ROWS, S::N1), idesc1w = tc::idesc_tf32(S::ROWS, 2 * S::N1);
  const bool warp0 = (threadIdx.x >> 5) == 0;
  bool ok = true;
  for (int ch = 0; ch < S::NCH; ++ch) {
    const int st = ch & 1;
    float2 vp[8], vh[8];
    form(ch, raw, vp, vh);
    if (ch + 1 < S::NCH) fetch(ch + 1, raw);
    // the stage is free once the MMAs of chunk ch - 2 are done; its next B1 chunk is then fetched
    if (warp0 && ch >= 2) {
      if (!bl.wait(2 + st, lim))
        *sflag = 1;
      else
        bl.copy(st, sR + (size_t)st * S::STAGE + 2 * S::ACH, mblock + (size_t)ch * 2 * S::BCH, B1_BYTES);
    }
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;
    if (!ok) break;
    float* stg = sR + (size_t)st * S::STAGE;
    float* aP = stg + (size_t)cl.side * S::ACH;        // parity of the P values this thread writes
    float* aH = stg + (size_t)(1 - cl.side) * S::ACH;  // parity of its H values
#pragma unroll
    for (int gq = 0; gq < 8; ++gq) {
#pragma unroll
      for (int cq = 0; cq < 2; ++cq) {
        const int comp = cq ^ cl.side;
        const int row = gq * 16 + cl.bt * 2 + comp;
        float hi, lo;
        tc::split_tf32(comp ? vp[gq].y : vp[gq].x, hi, lo);
        aP[tc::cm_index(row, cl.jl, S::KC)] = hi;
        aP[S::ROWS * S::KC + tc::cm_index(row, cl.jl, S::KC)] = lo;
        tc::split_tf32(comp ? vh[gq].y : vh[gq].x, hi, lo);
        aH[tc::cm_index(row, S::CJ + cl.jl, S::KC)] = hi;
        aH[S::ROWS * S::KC + tc::cm_index(row, S::CJ + cl.jl, S::KC)] = lo;
      }
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (warp0) {
      const bool good = bl.wait(st, lim);  // the same in every lane of warp 0
      if (!good) *sflag = 1;
      if (good) {
        const uint32_t sa = rbase + (uint32_t)(st * S::STAGE) * 4u;
        for (int par = 0; par < 2; ++par) {
          const uint32_t a_hi = sa + (uint32_t)(par * S::ACH) * 4u;
          const uint32_t a_lo = a_hi + (uint32_t)(S::ROWS * S::KC) * 4u;
          const uint32_t b_hi = sa + (uint32_t)(2 * S::ACH + par * S::BCH) * 4u;
          mma2_chunk(tbase + (uint32_t)(par * 2 * S::N1), a_hi, a_lo, b_hi, ch == 0, idesc1w, idesc1);
        }
      }
      bl.commit(2 + st);
    }
  }
  // the last chunk's commit covers every GEMM1 MMA
  if (ok) {
    bool w = warp0 ? bl.wait(2 + ((S::NCH - 1) & 1), lim) : true;
    ok = __syncthreads_and(w);
    tc::fence_after_sync();
    ok = ok && !*sflag;
  }
  return ok;
}

// The symmetric (side 0) or antisymmetric (side 1) sum of v with its value at
// the mirror latitude, held by lane ^ 16.
__device__ __forceinline__ float2 mirror_sum(float2 v, int side) {
  float2 o;
  o.x = __shfl_xor_sync(0xffffffffu, v.x, 16);
  o.y = __shfl_xor_sync(0xffffffffu, v.y, 16);
  return side ? csub(o, v) : cadd(v, o);
}

// D1 (both parities) -> staging res[g][n - m][member, re/im] for row groups g < ngroups
__device__ __forceinline__ void read_d1(uint32_t tbase, float* res, int ngroups, int C0, int C1) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = warp & 3, par = warp >> 2;
  const int row = quarter * 32 + lane;
  const int gq = row >> 4, btc = row & 15;
  const int Cp = par ? C1 : C0;
#pragma unroll
  for (int c0 = 0; c0 < S::N1; c0 += 16) {
    float v[16], v1[16];
    tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * par * S::N1 + c0), v);
    tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((2 * par + 1) * S::N1 + c0), v1);
    if (gq < ngroups) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int c = c0 + i;
        if (c < Cp) res[(gq * S::CNT + (par + 2 * c)) * 16 + btc] = v[i] + v1[i];
      }
    }
  }
}

// GEMM2 over the four units u = 2 par + half (128 x 80 x K2 each) into D2
// (TMEM columns [160 par, 160 par + 160)), B2 halves double-buffered (buffer
// u % 2).  Unit 0's copy into buffer 0 was issued before the epilogue; buffer 1
// (the D1 staging) is filled here.  Warp 0 only; false when a wait ran out.
__device__ __forceinline__ bool gemm2_halves(BarLog& bl, float* const* buf, const float* mblock, uint32_t a2base,
                                             int a2_floats, uint32_t tbase, uint32_t lim) {
  const uint32_t idesc2 = tc::idesc_tf32(S::ROWS, S::N2H);
  auto unit_mma = [&](int u) {
    const uint32_t a2 = a2base + (uint32_t)(2 * (u >> 1) * a2_floats) * 4u;
    const uint32_t bh = tc::smem_u32(buf[u & 1]);
    mma3<S::K2>(tbase + (uint32_t)((u >> 1) * S::N2 + (u & 1) * S::N2H), a2, a2 + (uint32_t)a2_floats * 4u, bh,
                bh + S::N2H * S::K2 * 4u, idesc2);
    bl.commit(6 + (u & 1));
  };
  // issue u0, u1; refill each buffer with the same half of parity 1 once its MMAs are done; issue u2, u3
  bl.copy(5, buf[1], mblock + S::B1 + S::B2H, B2_BYTES);
  bool good = bl.wait(4, lim);
  if (good) unit_mma(0);
  good = good && bl.wait(5, lim);
  if (good) unit_mma(1);
  good = good && bl.wait(6, lim);
  if (good) bl.copy(4, buf[0], mblock + S::B1 + 2 * S::B2H, B2_BYTES);
  good = good && bl.wait(7, lim);
  if (good) bl.copy(5, buf[1], mblock + S::B1 + 3 * S::B2H, B2_BYTES);
  good = good && bl.wait(4, lim);
  if (good) unit_mma(2);
  good = good && bl.wait(5, lim);
  if (good) unit_mma(3);
  return good && bl.wait(7, lim);  // the last commit covers every GEMM2 MMA
}

// D2 (both parities) -> output staging out[slot][member][j][re/im]: the P
// columns of row group q go to slot pslot(q), the H columns to hslot(q) (-1: none)
template <class PSlot, class HSlot>
__device__ __forceinline__ void read_d2(uint32_t tbase, float* out, PSlot pslot, HSlot hslot) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = warp & 3, half = warp >> 2;
  const int row = quarter * 32 + lane;
  const int q = row >> 4, btc = row & 15, bti = btc >> 1, comp = btc & 1;
  const bool hcols = half == 1;
  const int slot = hcols ? hslot(q) : pslot(q);
  const uint32_t lanes = (uint32_t)(quarter * 32) << 16;
#pragma unroll
  for (int cc = 0; cc < S::JH / 16; ++cc) {
    const int col0 = half * S::JH + cc * 16;
    float E[16], O[16];
    tc::tmem_ld16(tbase + lanes + (uint32_t)col0, E);
    tc::tmem_ld16(tbase + lanes + (uint32_t)(S::N2 + col0), O);
    if (slot >= 0) {
      float* o = out + (size_t)(slot * S::MT + bti) * S::OST + comp;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int jj = cc * 16 + i;
        o[2 * jj] = E[i] + O[i];
        o[2 * (S::J - 1 - jj)] = hcols ? (O[i] - E[i]) : (E[i] - O[i]);
      }
    }
  }
}
}  // namespace

size_t spec_tc106_smem_bytes() { return (size_t)(S::REGION + S::COEF) * sizeof(float) + 256; }
size_t spec_tc106_adj_smem_bytes() { return (size_t)(S::AREGION + S::COEF) * sizeof(float) + 256; }
size_t spec_tc106_basis_floats() { return (size_t)S::CNT * S::BLOCK; }

// Pack the FP64 basis of M = 106 into the per-m operand blocks: B1 as
// [chunk][par][hi, lo][N1][KC] (K = [P at the chunk's 16 j' | H at them]), B2
// as [par][half][hi, lo][N2H][K2].
__global__ void k_pack_tc106_basis(const double* __restrict__ Pw_f, const double* __restrict__ Hw_f,
                                   const double* __restrict__ P_i, const double* __restrict__ H_i,
                                   const int* __restrict__ boff, float* __restrict__ out) {
  const int m = blockIdx.x;
  const int cnt = S::CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  float* blk = out + (size_t)m * S::BLOCK;
  for (int i = threadIdx.x; i < S::BLOCK; i += blockDim.x) blk[i] = 0.f;
  __syncthreads();
  const int base = boff[m];
  for (int par = 0; par < 2; ++par) {
    const int Cp = par ? C1 : C0;
    const int poff = par ? S::JH * C0 : 0;
    for (int i = threadIdx.x; i < Cp * S::JH * 2; i += blockDim.x) {
      const int c = i / (2 * S::JH), r = i % (2 * S::JH);
      const bool hcol = r >= S::JH;
      const int jp = hcol ? r - S::JH : r;
      const int ch = jp / S::CJ, k = (hcol ? S::CJ : 0) + jp % S::CJ;
      const double v = hcol ? Hw_f[base + poff + jp * Cp + c] : Pw_f[base + poff + jp * Cp + c];
      float* bh = blk + (size_t)(ch * 2 + par) * S::BCH;
      const float hi = tc::to_tf32((float)v);
      bh[tc::cm_index(c, k, S::KC)] = hi;
      bh[S::N1 * S::KC + tc::cm_index(c, k, S::KC)] = tc::to_tf32((float)(v - (double)hi));
    }
    for (int i = threadIdx.x; i < S::N2 * Cp; i += blockDim.x) {
      const int col = i / Cp, c = i % Cp, jp = col % S::JH;
      const double v = (col < S::JH) ? P_i[base + poff + c * S::JH + jp] : H_i[base + poff + c * S::JH + jp];
      const int half = col / S::N2H, hc = col % S::N2H;
      float* bh = blk + S::B1 + (size_t)(par * 2 + half) * S::B2H;
      const float hi = tc::to_tf32((float)v);
      bh[tc::cm_index(hc, c, S::K2)] = hi;
      bh[S::N2H * S::K2 + tc::cm_index(hc, c, S::K2)] = tc::to_tf32((float)(v - (double)hi));
    }
  }
}

// The forward kernel contracts with the weighted forward basis and the inverse
// basis; the adjoint with the unweighted basis in the forward layout
// (transposed inverse Legendre) and the weighted one in the inverse layout
// (transposed forward Legendre).
int pack_tc106_basis(const GroupGeom& gg, float* out, bool adjoint, cudaStream_t s) {
  if (gg.M != S::M || gg.J != S::J) return SWP_ERR_ARG;
  if (adjoint)
    k_pack_tc106_basis<<<S::CNT, 256, 0, s>>>(gg.b64[B_P_F], gg.b64[B_H_F], gg.b64[B_PW_I], gg.b64[B_HW_I], gg.boff,
                                              out);
  else
    k_pack_tc106_basis<<<S::CNT, 256, 0, s>>>(gg.b64[B_PW_F], gg.b64[B_HW_F], gg.b64[B_P_I], gg.b64[B_H_I], gg.boff,
                                              out);
  return cudaGetLastError() == cudaSuccess ? SWP_OK : SWP_ERR_CUDA;
}

__global__ void __launch_bounds__(256, 1) k_spectral_tc106(const __grid_constant__ SpecLaunch<float> L,
                                                           const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NSPX = SlotCount<float>::NP;
  constexpr int NSLOT = NSPX + NSH;
  constexpr int MT = S::MT, J = S::J, CNT = S::CNT;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  pdl_enter();
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const StepCfg& cfg = L.cfg;
  const int m = idx / G.ntb;
  const int b0 = (idx % G.ntb) * MT;
  const int mt = min(MT, G.B - b0);
  const int cnt = CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  const size_t FS = (size_t)CNT * G.B * J;
  const bool incr = cfg.incremental != 0;
  if (cfg.scheme != 0 || L.mode != 0) {  // the host launches this kernel for modified-Euler steps only
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const float* mblock = basis.p[gi] + (size_t)m * S::BLOCK;

  float* sR = (float*)smem_raw;            // GEMM1 stages | A2, D1 staging, GEMM2 buffers | output staging
  float* sig = sR + S::REGION;             // [MT][CNT] x 5
  float* sigP = sig + MT * CNT;
  float* sigm1 = sigP + MT * CNT;
  float* sigPm1 = sigm1 + MT * CNT;
  float* tcmn = sigPm1 + MT * CNT;
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + MT * CNT) + 15) & ~(uintptr_t)15);  // [8]
  uint32_t* tslot = (uint32_t*)(mbar + BarLog::NB);
  int* sflag = (int*)(tslot + 1);
  int* sdead = sflag + 1;                  // [MT]
  BarLog bl(mbar);                         // used by warp 0

  // chunk inputs of the thread: the 11 Fourier fields step_combos_ld reads
  // (eta, delta, Phi, A..G) and the step factors at (member, j)
  const ChunkLane cl;
  struct Raw {
    T2 v[11];
    StepCoefs<T> kc;
  } raw;
  auto fetch = [&](int ch, Raw& r) {
    const int jp = ch * S::CJ + cl.jl;
    const int j = cl.side ? (J - 1 - jp) : jp;
    if (cl.bt < mt) {
      const int b = b0 + cl.bt;
      const size_t o = ((size_t)m * G.B + b) * J + j;
#pragma unroll
      for (int q = 0; q < 11; ++q) r.v[q] = G.four[(size_t)field106(q) * FS + o];
      r.kc = load_step_coefs<T>(G, b, j);
    }
  };
  auto form = [&](int ch, const Raw& r, T2* vp, T2* vh) {
    T2 c[NSLOT];
    if (cl.bt < mt) {
      const int jp = ch * S::CJ + cl.jl;
      const int j = cl.side ? (J - 1 - jp) : jp;
      step_combos_ld<T>(G, cfg, 0, incr, m, b0 + cl.bt, j, [&](int f) { return r.v[slot106(f)]; }, c, &r.kc);
    } else {
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) c[q] = mk<T2>(0, 0);
    }
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) c[q] = mirror_sum(c[q], cl.side);
#pragma unroll
    for (int gq = 0; gq < 8; ++gq) {
      vp[gq] = c[group_p106(gq)];
      vh[gq] = group_h106(gq) >= 0 ? c[NSPX + group_h106(gq)] : mk<T2>(0, 0);
    }
  };

  // ---- phase 0: barriers, the first two B1 chunks, TMEM; chunk 0's inputs;
  // coefficients; blow-up gate
  setup_chunks(bl, sR, mblock, tslot, sflag);
  fetch(0, raw);
  load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, MT, cnt, CNT, sig, sigP, sigm1, sigPm1, tcmn);
  if (threadIdx.x < MT) {
    const int bt = threadIdx.x;
    int dead = 0;
    if (bt < mt && cfg.diagnostics) {
      const int b = b0 + bt;
      const double rms = sqrt(G.diag[((size_t)cfg.step * NDIAG + D_RMS2) * G.B + b]);
      dead = (G.member[MS_DEAD * G.B + b] != 0.0) || (rms > cfg.blowup);
      if (m == 0) {
        G.member[MS_DEAD * G.B + b] = dead ? 1.0 : 0.0;
        G.diag[((size_t)cfg.step * NDIAG + D_DEAD) * G.B + b] = dead ? 1.0 : 0.0;
      }
    }
    sdead[bt] = dead;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  // ---- phase 1: GEMM1 over the latitude chunks
  bool ok = gemm1_chunks(bl, sR, mblock, tbase, sflag, basis.wait_limit, cl, raw, fetch, form);

  // post-GEMM1 layout
  float* sA2 = sR;
  float* sRes = sR + S::OFF_RES;
  float* buf[2] = {sR + S::OFF_BUF0, sR + S::OFF_RES};
  // write-out: thread -> member wbt, latitudes wj, wj + 1 (16-byte accesses)
  int wbt[S::NWPAIR], wj[S::NWPAIR];
#pragma unroll
  for (int k = 0; k < S::NWPAIR; ++k) {
    const int q = threadIdx.x + 256 * k;
    wbt[k] = q < MT * J / 2 ? q / (J / 2) : MT;
    wj[k] = 2 * (q % (J / 2));
  }
  T2 pold[S::NWPAIR][3][2], pmid[S::NWPAIR][3][2];
  T wal[S::NWPAIR], wan[S::NWPAIR];
  if (ok) {
    // B2 (parity 0, column half 0) into buffer 0, overlapped with the epilogue
    if (threadIdx.x < 32) bl.copy(4, buf[0], mblock + S::B1, B2_BYTES);
    // ---- phase 2: D1 -> staging sRes[g][n-m][member, re/im]; zero the A2 operands
    read_d1(tbase, sRes, 8, C0, C1);
    for (int i = threadIdx.x; i < 4 * S::A2; i += blockDim.x) sA2[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 3: spectral epilogue -> A2 operands [par][hi, lo][112 rows][K2]
    for (int t = threadIdx.x; t < MT * cnt; t += blockDim.x) {
      const int bti = t % MT, kk = t / MT, n = m + kk;
      const int par = kk & 1, cc = kk >> 1;
      const T s = sig[bti * CNT + kk], sp = sigP[bti * CNT + kk], tcv = tcmn[bti * CNT + kk];
      const T sm1 = sigm1[bti * CNT + kk], spm1 = sigPm1[bti * CNT + kk];
      const T nn1 = (T)(n * (n + 1));
      const T om = bti < mt ? G.mco[MC_OM * G.B + b0 + bti] : (T)0;
      T kv[7][2];
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        auto R = [&](int gq) { return sRes[(gq * CNT + kk) * 16 + bti * 2 + comp]; };
        const T sphi = R(0) + nn1 * R(1);
        const T sdel = R(2) + nn1 * R(3);
        const T seta = R(4);
        T cdel, ceta, kphi, kdel, keta;
        if (incr) {
          // new = curr + Inv(dc), dc = (sigma - 1) Fwd(curr) + sigma * tendency
          const T iphi = R(5), idel = R(6), ieta = R(7);
          cdel = s * (idel + sdel);
          ceta = s * (ieta + seta);
          kphi = spm1 * iphi + sp * sphi;
          kdel = sm1 * idel + s * sdel;
          keta = sm1 * ieta + s * seta;
        } else {
          kphi = sp * sphi;
          cdel = s * sdel;
          ceta = s * seta;
          kdel = cdel;
          keta = ceta;
        }
        const T dp = (n == 0) ? (T)0 : cdel;
        T ep = (n == 0) ? (T)0 : ceta;
        if (m == 0 && n == 1 && comp == 0) ep -= om;
        kv[0][comp] = keta;
        kv[1][comp] = kdel;
        kv[2][comp] = kphi;
        kv[5][comp] = ep * tcv;    // eta_s, H input of U
        kv[6][comp] = -dp * tcv;   // -delta_s, H input of V
      }
      // Uprep = -i m delta_s, Vprep = -i m eta_s
      const T xm = (T)m;
      kv[3][0] = -xm * kv[6][1];
      kv[3][1] = xm * kv[6][0];
      kv[4][0] = xm * kv[5][1];
      kv[4][1] = -xm * kv[5][0];
      float* aH = sA2 + (size_t)(2 * par) * S::A2;
      float* aL = aH + S::A2;
#pragma unroll
      for (int q = 0; q < 7; ++q)
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = q * 16 + bti * 2 + comp;
          float hi, lo;
          tc::split_tf32(kv[q][comp], hi, lo);
          aH[tc::cm_index(row, cc, S::K2)] = hi;
          aL[tc::cm_index(row, cc, S::K2)] = lo;
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- phase 4: GEMM2 (rows 112..127 read past the A2 operands and are
    // ignored); the write-out inputs are loaded meanwhile
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k) {
      wal[k] = (T)0;
      wan[k] = (T)0;
      if (wbt[k] < mt) {
        load_step_rows<T>(G, cfg, incr, FS, ((size_t)m * G.B + b0 + wbt[k]) * J + wj[k], pold[k], pmid[k]);
        wal[k] = G.mco[(cfg.raw ? MC_RAWM : MC_ALPHA) * G.B + b0 + wbt[k]];
        wan[k] = cfg.raw ? G.mco[MC_RAWN * G.B + b0 + wbt[k]] : (T)0;
      }
    }
    if (threadIdx.x < 32 && !gemm2_halves(bl, buf, mblock, tc::smem_u32(sA2), S::A2, tbase, basis.wait_limit))
      *sflag = 1;
    ok = __syncthreads_and(!*sflag);
    tc::fence_after_sync();
  }
  if (ok) {
    // ---- phase 5: D2 -> output staging Out[f][member][j][re/im]; f 0..4 from the P
    // columns of rows q 0..4, f 5, 6 from the H columns of rows q 5, 6
    float* Out = sR;
    read_d2(tbase, Out, [](int q) { return q <= 4 ? q : -1; }, [](int q) { return (q == 5 || q == 6) ? q : -1; });
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 6: write-out and carries, by latitude pairs
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k) {
      if (wbt[k] < mt && !sdead[wbt[k]]) {
        const size_t o = ((size_t)m * G.B + b0 + wbt[k]) * J + wj[k];
        auto get = [&](int f, int e) {
          return *(const float2*)&Out[(size_t)(f * MT + wbt[k]) * S::OST + 2 * (wj[k] + e)];
        };
        T2 nw[3][2], uu[2], vv[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          nw[0][e] = get(0, e);
          nw[1][e] = get(1, e);
          nw[2][e] = get(2, e);
          uu[e] = cadd(get(3, e), get(5, e));
          vv[e] = cadd(get(4, e), get(6, e));
        }
        store_step_rows<T>(G, cfg, incr, FS, o, wal[k], wan[k], nw, cfg.test != 1, uu, vv, pold[k], pmid[k]);
      }
    }
    if (m == 0 && threadIdx.x < mt && !sdead[threadIdx.x]) {
      const int b = b0 + threadIdx.x;
      double wc = G.member[MS_WCURR * G.B + b], wm = G.member[MS_WMID * G.B + b];
      step_residual_weights(cfg, G.par[P_ALPHA * G.B + b], G.par[P_WALPHA * G.B + b], wc, wm);
      G.member[MS_WMID * G.B + b] = wm;
      G.member[MS_WCURR * G.B + b] = wc;
      G.member[MS_UPDATED * G.B + b] = 1.0;
    }
  } else if (threadIdx.x < 32) {
    // a wait ran out: report, then drain (bounded) what this CTA issued before freeing TMEM
    if (threadIdx.x == 0) atomicExch(err, 1);
    bl.drain();
  }
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tbase, S::TMEM_COLS);
}

// Adjoint of k_spectral_tc106 (modified Euler), the chunked form of
// k_spectral_adj_tc:
//   GEMM1' (transposed inverse Legendre), per parity, over the latitude chunks:
//     row = group q (7: lambda of eta, delta, Phi, Uprep, Vprep on P; of U, V on
//     H; group 7 zero) x member x re/im, k = [P at j' | H at j'] (unweighted)
//   epilogue: transposed wind inversion, n(n+1), hyperdiffusion, incremental form
//   GEMM2' (transposed forward Legendre), per parity and column half:
//     row = slot q (8: PhiP1, PhiP2, dP1, dP2, eP1, identity Phi, delta, eta)
//     x member x re/im, col = [Pw at j' | Hw at j']; the Hw columns of slots 0,
//     2, 3, 4 are the H slots PhiH1, dH1, dH2, eH1
//   write-out: adj_store_rows (transposed combination) + Phibar gradient.
__global__ void __launch_bounds__(256, 1) k_spectral_adj_tc106(const __grid_constant__ SpecLaunch<float> L,
                                                               const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NKADJ = 8;
  constexpr int MT = S::MT, J = S::J, JH = S::JH, CNT = S::CNT;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  pdl_enter();
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const StepCfg& cfg = L.cfg;
  const int m = idx / G.ntb;
  const int b0 = (idx % G.ntb) * MT;
  const int mt = min(MT, G.B - b0);
  const int cnt = CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  const size_t FS = (size_t)CNT * G.B * J;
  const bool incr = cfg.incremental != 0;
  if (cfg.scheme != 0) {  // the host launches this kernel for modified-Euler steps only
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const float* mblock = basis.p[gi] + (size_t)m * S::BLOCK;

  float* sR = (float*)smem_raw;            // GEMM1' stages | A2', D1' staging, GEMM2' buffers | output staging
  float* sig = sR + S::AREGION;
  float* sigP = sig + MT * CNT;
  float* sigm1 = sigP + MT * CNT;
  float* sigPm1 = sigm1 + MT * CNT;
  float* tcmn = sigPm1 + MT * CNT;
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + MT * CNT) + 15) & ~(uintptr_t)15);  // [8]
  uint32_t* tslot = (uint32_t*)(mbar + BarLog::NB);
  int* sflag = (int*)(tslot + 1);
  BarLog bl(mbar);

  // chunk inputs of the thread: lambda_Y of eta, delta, Phi, Uprep, Vprep at (member, j)
  const ChunkLane cl;
  struct Raw {
    T2 y[5];
  } raw;
  auto fetch = [&](int ch, Raw& r) {
    const int jp = ch * S::CJ + cl.jl;
    const int j = cl.side ? (J - 1 - jp) : jp;
    const size_t o = ((size_t)m * G.B + b0 + cl.bt) * J + j;
#pragma unroll
    for (int f = 0; f < 5; ++f) r.y[f] = cl.bt < mt ? G.lamY[(size_t)f * FS + o] : mk<T2>(0, 0);
  };
  // lambda_Y of eta, delta, Phi, Uprep, Vprep on the P columns, of U, V on the H columns
  auto form = [&](int, const Raw& r, T2* vp, T2* vh) {
    T2 y[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) y[f] = mirror_sum(r.y[f], cl.side);
#pragma unroll
    for (int gq = 0; gq < 8; ++gq) {
      vp[gq] = gq < 5 ? y[gq] : mk<T2>(0, 0);
      vh[gq] = (gq == 5 || gq == 6) ? y[gq - 2] : mk<T2>(0, 0);
    }
  };

  // ---- phase 0: barriers, the first two B1' chunks, TMEM; chunk 0's inputs; coefficients
  setup_chunks(bl, sR, mblock, tslot, sflag);
  fetch(0, raw);
  load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, MT, cnt, CNT, sig, sigP, sigm1, sigPm1, tcmn);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  // ---- phase 1: GEMM1' over the latitude chunks
  bool ok = gemm1_chunks(bl, sR, mblock, tbase, sflag, basis.wait_limit, cl, raw, fetch, form);

  float* sA2 = sR;
  float* sRes = sR + S::AOFF_RES;
  float* buf[2] = {sR + S::AOFF_BUF0, sR + S::AOFF_RES};
  int wbt[S::NWPAIR], wj[S::NWPAIR];
#pragma unroll
  for (int k = 0; k < S::NWPAIR; ++k) {
    const int q = threadIdx.x + 256 * k;
    wbt[k] = q < MT * J / 2 ? q / (J / 2) : MT;
    wj[k] = 2 * (q % (J / 2));
  }
  AdjRowsIn<T> pin[S::NWPAIR];  // write-out inputs, loaded ahead of GEMM2'
  if (ok) {
    if (threadIdx.x < 32) bl.copy(4, buf[0], mblock + S::B1, B2_BYTES);
    // ---- phase 2: D1' -> sRes[q][n-m][member, re/im] (7 groups); zero the A2' operands
    read_d1(tbase, sRes, 7, C0, C1);
    for (int i = threadIdx.x; i < 4 * S::AA2; i += blockDim.x) sA2[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 3: transposed wind inversion, n(n+1), hyperdiffusion -> A2' [par][hi, lo][128][K2]
    for (int t = threadIdx.x; t < MT * cnt; t += blockDim.x) {
      const int bti = t % MT, kk = t / MT, n = m + kk;
      const int par = kk & 1, c = kk >> 1;
      auto R = [&](int q, int comp) { return sRes[(q * CNT + kk) * 16 + bti * 2 + comp]; };
      const T xm = (T)m;
      const T tcv = tcmn[bti * CNT + kk];
      const T s = sig[bti * CNT + kk], sp = sigP[bti * CNT + kk];
      const T sm1 = sigm1[bti * CNT + kk], spm1 = sigPm1[bti * CNT + kk];
      const T nn1 = (T)(n * (n + 1));
      // lambda delta_s = (i m) lambda Uprep - lambda Hin_V ; lambda eta_s = (i m) lambda Vprep + lambda Hin_U
      const T lds_r = -xm * R(3, 1) - R(6, 0), lds_i = xm * R(3, 0) - R(6, 1);
      const T les_r = -xm * R(4, 1) + R(5, 0), les_i = xm * R(4, 0) + R(5, 1);
      const T w = (n == 0) ? (T)0 : tcv;
      const T lce_r = R(0, 0) + w * les_r, lce_i = R(0, 1) + w * les_i;
      const T lcd_r = R(1, 0) + w * lds_r, lcd_i = R(1, 1) + w * lds_i;
      const T lcp_r = R(2, 0), lcp_i = R(2, 1);
      T kv[NKADJ][2];
      kv[0][0] = sp * lcp_r; kv[0][1] = sp * lcp_i;
      kv[1][0] = nn1 * sp * lcp_r; kv[1][1] = nn1 * sp * lcp_i;
      kv[2][0] = s * lcd_r; kv[2][1] = s * lcd_i;
      kv[3][0] = nn1 * s * lcd_r; kv[3][1] = nn1 * s * lcd_i;
      kv[4][0] = s * lce_r; kv[4][1] = s * lce_i;
      kv[5][0] = incr ? spm1 * R(2, 0) : (T)0; kv[5][1] = incr ? spm1 * R(2, 1) : (T)0;
      kv[6][0] = incr ? (s * w * lds_r + sm1 * R(1, 0)) : (T)0; kv[6][1] = incr ? (s * w * lds_i + sm1 * R(1, 1)) : (T)0;
      kv[7][0] = incr ? (s * w * les_r + sm1 * R(0, 0)) : (T)0; kv[7][1] = incr ? (s * w * les_i + sm1 * R(0, 1)) : (T)0;
      float* aH = sA2 + (size_t)(2 * par) * S::AA2;
      float* aL = aH + S::AA2;
#pragma unroll
      for (int q = 0; q < NKADJ; ++q)
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = q * 16 + bti * 2 + comp;
          float hi, lo;
          tc::split_tf32(kv[q][comp], hi, lo);
          aH[tc::cm_index(row, c, S::K2)] = hi;
          aL[tc::cm_index(row, c, S::K2)] = lo;
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- phase 4: GEMM2'; write-out inputs loaded meanwhile
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k)
      if (wbt[k] < mt) adj_load_rows<T>(G, incr, FS, ((size_t)m * G.B + b0 + wbt[k]) * J + wj[k], pin[k]);
    if (threadIdx.x < 32 && !gemm2_halves(bl, buf, mblock, tc::smem_u32(sA2), S::AA2, tbase, basis.wait_limit))
      *sflag = 1;
    ok = __syncthreads_and(!*sflag);
    tc::fence_after_sync();
  }
  if (ok) {
    // ---- phase 5: D2' -> output staging Out[slot][member][j][re/im]: slots 0..7
    // from the Pw columns of rows q, slots 8..11 from the Hw columns of rows 0, 2, 3, 4
    float* Out = sR;
    read_d2(tbase, Out, [](int q) { return q; },
            [](int q) { return adj_hslot106(q) >= 0 ? NKADJ + adj_hslot106(q) : -1; });
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 6: transposed combination -> lambda of the state fields; the
    // Phibar gradient terms of each latitude pair go to sgp
    float* sgp = sR + S::AOFF_GP;  // [MT][J / 2]
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k) {
      if (wbt[k] < mt) {
        const int b = b0 + wbt[k];
        const size_t o = ((size_t)m * G.B + b) * J + wj[k];
        auto ld = [&](int q, int e) {
          return *(const float2*)&Out[(size_t)(q * MT + wbt[k]) * S::OST + 2 * (wj[k] + e)];
        };
        const T gp = adj_store_rows<T, NKADJ>(G, cfg, incr, FS, o, m, b, wj[k], ld, pin[k]);
        sgp[wbt[k] * JH + wj[k] / 2] = gp;
      }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (G.grad && warp < mt) {  // one warp per member, reduced in a fixed order
      float acc = 0.f;
      for (int i = lane; i < JH; i += 32) acc += sgp[warp * JH + i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) atomicAdd(&G.grad[G_PHIBAR * G.B + b0 + warp], (double)acc);
    }
  } else if (threadIdx.x < 32) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    bl.drain();
  }
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tbase, S::TMEM_COLS);
}

void spec_tc106_set_attributes() {
  cudaFuncSetAttribute(k_spectral_tc106, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_tc106_smem_bytes());
  cudaFuncSetAttribute(k_spectral_adj_tc106, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)spec_tc106_adj_smem_bytes());
}

cudaError_t launch_spec_tc106(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                              cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  cudaError_t e = launch_pdl(k_spectral_tc106, nblocks, 256, spec_tc106_smem_bytes(), s, true, L, basis, err);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_spec_adj_tc106(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                                  cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  cudaError_t e = launch_pdl(k_spectral_adj_tc106, nblocks, 256, spec_tc106_adj_smem_bytes(), s, true, L, basis, err);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace swp
