// Tensor-core (tcgen05) Legendre sandwich of one modified-Euler step, FP32
// fast path, truncation M = 42 (64 x 128 Gauss grid).
//
// Same per-m decomposition and arithmetic as k_spectral (spectral.cu), with the
// two contractions issued as kind::tf32 MMAs in 3xTF32 split precision
// (a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accumulation in TMEM):
//   GEMM1, forward Legendre, once per parity of n - m:
//     D1[row, c] = sum_k A1[row, k] B1[c, k]
//     row = group g (8) x member (8) x re/im (2) = 128,
//     k = [Pw at j' (32) | Hw at j' (32)], c -> n = m + par + 2c (N = 32)
//   epilogue in shared memory: n(n+1), hyperdiffusion, the incremental form,
//     wind-inversion inputs (spectral_transform.py:577-594, filters.py:95-151)
//   GEMM2, inverse Legendre, once per parity:
//     D2[row, col] = sum_c A2[row, c] B2[col, c]
//     row = input q (7) x member (8) x re/im (2) = 112 (of the 128 MMA rows),
//     col = [P at j' (32) | H at j' (32)]
// The forward groups are the combined inputs of step_combos paired as
//   g0 (PhiP1 | PhiH1)  g1 (PhiP2 | 0)  g2 (dP1 | dH1)  g3 (dP2 | dH2)
//   g4 (eP1 | eH1)      g5..g7 (curr Phi, delta, eta | 0)
// so that one row of D1 is already the sum of its P and H contractions.
// The basis blocks of each m are packed once per plan (TF32 hi/lo split of the
// FP64 basis, core-matrix layout) and fetched with bulk (TMA) copies.  Every
// wait is bounded: on a timeout the CTA sets the device error word, waits
// (bounded) for what it issued, frees its TMEM and returns.
#include "swp_internal.h"
#include "spec_common.cuh"
#include "tc_common.cuh"

namespace swp {

namespace {
constexpr int TC_M = 42, TC_J = 64, TC_JH = 32;
constexpr int TC_MT = 8;                           // members per CTA
constexpr int TC_CNT = TC_M + 1;                   // n = m..M, at most 43
constexpr int TC_ROWS = 128;                       // MMA M
constexpr int TC_K1 = 2 * TC_JH;                   // 64
constexpr int TC_N1 = 32;                          // >= ceil(43 / 2), multiple of 16
constexpr int TC_R2 = 112;                         // used rows of GEMM2
constexpr int TC_K2 = 24;                          // >= ceil(43 / 2), multiple of 8
constexpr int TC_N2 = 2 * TC_JH;                   // 64
constexpr int TC_B1 = 4 * TC_N1 * TC_K1;           // [par][hi, lo][N1][K1] = 8192 floats
constexpr int TC_B2 = 4 * TC_N2 * TC_K2;           // [par][hi, lo][N2][K2] = 6144 floats
constexpr int TC_BLOCK = TC_B1 + TC_B2;            // packed basis floats per m
constexpr int TC_A = 2 * TC_ROWS * TC_K1;          // A region: 16384 floats (64 KB)
constexpr int TC_A2 = TC_R2 * TC_K2;               // one A2 operand (2688 floats)
constexpr int TC_RES0 = 4 * TC_A2;                 // D1 staging inside the A region
constexpr int TC_RES = 8 * TC_CNT * 16;            // [g][n-m][member, re/im]
constexpr int TC_OST = 2 * TC_J + 2;               // output staging row stride (floats)
constexpr int TC_NOUT = 7;                         // eta, delta, Phi, Uprep, Vprep | U_H, V_H
constexpr int TC_COEF = 5 * TC_MT * TC_CNT;
constexpr int TC_TMEM_COLS = 256;                  // D1: 2 x (2 x 32), D2: 2 x 64 (D2 reuses D1's columns)
static_assert(TC_RES0 + TC_RES <= TC_A, "D1 staging must fit in the A region");
static_assert(TC_NOUT * TC_MT * TC_OST <= TC_A, "output staging must fit in the A region");
// the MMA reads all 128 rows of the last A2 operand: they must stay in the A region
static_assert(3 * TC_A2 + TC_ROWS * TC_K2 <= TC_A, "A2 over-read must stay in the A region");
static_assert(TC_B2 <= TC_B1, "B2 reuses the B1 buffer");
// inputs of a modified-Euler step, staged by bulk copies at the start of the A region
constexpr int TC_NIN = 11;
static_assert(TC_NIN * TC_MT * TC_J * 2 <= TC_A, "staged inputs must fit in the A region");
__host__ __device__ constexpr int stage_field(int q) {  // staged slot -> Fourier field
  return q == 0 ? F_ETA : q == 1 ? F_DELTA : q == 2 ? F_PHI : F_A + (q - 3);
}
// Fourier field -> staged slot, for the fields stage_field covers (F_A..F_G are
// consecutive); any other field is never read by the modified-Euler combination
__host__ __device__ constexpr int stage_slot(int f) {
  return f == F_ETA ? 0 : f == F_DELTA ? 1 : f == F_PHI ? 2 : (f >= F_A && f <= F_G) ? f - F_A + 3 : 0;
}
static_assert(F_G - F_A + 4 == TC_NIN, "staged fields");

// slots of forward group g (compile-time, so that the slot arrays stay in registers)
__host__ __device__ constexpr int group_p(int g) {
  return g == 0 ? SP_PHI1 : g == 1 ? SP_PHI2 : g == 2 ? SP_D1 : g == 3 ? SP_D2 : g == 4 ? SP_E1
       : g == 5 ? SP_IPHI : g == 6 ? SP_ID : SP_IE;
}
__host__ __device__ constexpr int group_h(int g) {
  return g == 0 ? SH_PHI1 : g == 2 ? SH_D1 : g == 3 ? SH_D2 : g == 4 ? SH_E1 : -1;
}
}  // namespace

size_t spec_tc_smem_bytes() { return (size_t)(TC_A + TC_B1 + TC_COEF) * sizeof(float) + 256; }
size_t spec_tc_basis_floats() { return (size_t)TC_CNT * TC_BLOCK; }
int spec_tc_members_per_cta() { return TC_MT; }
bool spec_tc_supported(int M) { return M == TC_M; }

// Pack the FP64 basis of M = 42 into the per-m GEMM operand blocks.
__global__ void k_pack_tc_basis(const double* __restrict__ Pw_f, const double* __restrict__ Hw_f,
                                const double* __restrict__ P_i, const double* __restrict__ H_i,
                                const int* __restrict__ boff, float* __restrict__ out) {
  const int m = blockIdx.x;
  const int cnt = TC_CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  float* blk = out + (size_t)m * TC_BLOCK;
  for (int i = threadIdx.x; i < TC_BLOCK; i += blockDim.x) blk[i] = 0.f;
  __syncthreads();
  const int base = boff[m];
  for (int par = 0; par < 2; ++par) {
    const int Cp = par ? C1 : C0;
    const int poff = par ? TC_JH * C0 : 0;
    float* b1h = blk + (size_t)(2 * par) * TC_N1 * TC_K1;
    float* b1l = b1h + TC_N1 * TC_K1;
    float* b2h = blk + TC_B1 + (size_t)(2 * par) * TC_N2 * TC_K2;
    float* b2l = b2h + TC_N2 * TC_K2;
    for (int i = threadIdx.x; i < Cp * TC_K1; i += blockDim.x) {
      const int c = i / TC_K1, k = i % TC_K1, jp = k % TC_JH;
      const double v = (k < TC_JH) ? Pw_f[base + poff + jp * Cp + c] : Hw_f[base + poff + jp * Cp + c];
      const float hi = tc::to_tf32((float)v);
      b1h[tc::cm_index(c, k, TC_K1)] = hi;
      b1l[tc::cm_index(c, k, TC_K1)] = tc::to_tf32((float)(v - (double)hi));
    }
    for (int i = threadIdx.x; i < TC_N2 * Cp; i += blockDim.x) {
      const int col = i / Cp, c = i % Cp, jp = col % TC_JH;
      const double v = (col < TC_JH) ? P_i[base + poff + c * TC_JH + jp] : H_i[base + poff + c * TC_JH + jp];
      const float hi = tc::to_tf32((float)v);
      b2h[tc::cm_index(col, c, TC_K2)] = hi;
      b2l[tc::cm_index(col, c, TC_K2)] = tc::to_tf32((float)(v - (double)hi));
    }
  }
}

int pack_tc_basis(const GroupGeom& gg, float* out, cudaStream_t s) {
  if (gg.M != TC_M || gg.J != TC_J) return SWP_ERR_ARG;
  k_pack_tc_basis<<<TC_CNT, 256, 0, s>>>(gg.b64[B_PW_F], gg.b64[B_HW_F], gg.b64[B_P_I], gg.b64[B_H_I], gg.boff, out);
  return cudaGetLastError() == cudaSuccess ? SWP_OK : SWP_ERR_CUDA;
}

// The adjoint's operand blocks: GEMM1' contracts with the unweighted basis in
// the forward layout (transposed inverse Legendre), GEMM2' with the weighted
// basis in the inverse layout (transposed forward Legendre).
int pack_tc_basis_adj(const GroupGeom& gg, float* out, cudaStream_t s) {
  if (gg.M != TC_M || gg.J != TC_J) return SWP_ERR_ARG;
  k_pack_tc_basis<<<TC_CNT, 256, 0, s>>>(gg.b64[B_P_F], gg.b64[B_H_F], gg.b64[B_PW_I], gg.b64[B_HW_I], gg.boff, out);
  return cudaGetLastError() == cudaSuccess ? SWP_OK : SWP_ERR_CUDA;
}

namespace {
// the three products of one 3xTF32 K-sweep into d_tmem (K a multiple of 8)
__device__ __forceinline__ void mma_3xtf32(uint32_t d_tmem, uint32_t aH, uint32_t aL, uint32_t bH, uint32_t bL, int K,
                                           uint32_t idesc) {
  const uint32_t sbo = (uint32_t)(K / 4) * 128u;
  for (int kk = 0; kk < K / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32(d_tmem, tc::make_desc(aH + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc, kk > 0);
    tc::mma_tf32(d_tmem, tc::make_desc(aH + off, 128, sbo), tc::make_desc(bL + off, 128, sbo), idesc, 1);
    tc::mma_tf32(d_tmem, tc::make_desc(aL + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc, 1);
  }
}
// The same K-sweep in two MMAs per K-step.  The issue of an MMA, not its
// arithmetic, is what the narrow (N = 32) GEMM1 waits on, so a_hi is applied
// to b_hi and b_lo in one MMA of width 2n (the lo tile follows the hi tile in
// shared memory: rows n..2n-1 of that operand), giving d[0, n) = a_hi b_hi and
// d[n, 2n) = a_hi b_lo; a_lo b_hi then accumulates onto d[n, 2n).  The product
// is d[0, n) + d[n, 2n).  idesc_2n / idesc_n describe the 128 x 2n / 128 x n MMAs.
__device__ __forceinline__ void mma_3xtf32_2(uint32_t d_tmem, uint32_t aH, uint32_t aL, uint32_t bH, int n, int K,
                                             uint32_t idesc_2n, uint32_t idesc_n) {
  const uint32_t sbo = (uint32_t)(K / 4) * 128u;
  for (int kk = 0; kk < K / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32(d_tmem, tc::make_desc(aH + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc_2n, kk > 0);
    tc::mma_tf32(d_tmem + (uint32_t)n, tc::make_desc(aL + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc_n,
                 1);
  }
}
// the hi tile of a [hi, lo][N][K] operand pair is followed by its lo tile at (N / 8) stride offsets
static_assert(TC_N1 * TC_K1 * 4 == (TC_N1 / 8) * (TC_K1 / 4) * 128, "B1 lo tile must follow its hi tile");
}  // namespace

__global__ void __launch_bounds__(256, 2) k_spectral_tc(const __grid_constant__ SpecLaunch<float> L,
                                                        const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NSPX = SlotCount<float>::NP;
  constexpr int NSLOT = NSPX + NSH;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const float* gbasis = basis.p[gi];
  const StepCfg& cfg = L.cfg;
  const int J = TC_J;
  const int m = idx / G.ntb;
  const int b0 = (idx % G.ntb) * TC_MT;
  const int mt = min(TC_MT, G.B - b0);
  const int cnt = TC_CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  const size_t FS = (size_t)TC_CNT * G.B * J;
  const bool incr = cfg.incremental != 0;
  if (cfg.scheme != 0 || L.mode != 0) {  // the host launches this kernel for modified-Euler steps only
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }

  float* sA = (float*)smem_raw;            // staged inputs | A1 | A2 + D1 staging | output staging
  float* sB = sA + TC_A;                   // B1, then B2
  float* sRes = sA + TC_RES0;
  float* sig = sB + TC_B1;                 // [MT][CNT] x 5
  float* sigP = sig + TC_MT * TC_CNT;
  float* sigm1 = sigP + TC_MT * TC_CNT;
  float* sigPm1 = sigm1 + TC_MT * TC_CNT;
  float* tcmn = sigPm1 + TC_MT * TC_CNT;
  // [4]: 0 basis copies, 1 GEMM1 commits, 2 GEMM2 commit, 3 input copies
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + TC_MT * TC_CNT) + 15) & ~(uintptr_t)15);
  uint32_t* tslot = (uint32_t*)(mbar + 4);
  int* sflag = (int*)(tslot + 1);
  int* sdead = sflag + 1;                  // [MT]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // what thread 0 has issued, for the bounded drain on failure
  int n_tma = 0, n_in = 0, n_c1 = 0, n_c2 = 0;

  // ---- phase 0: barriers; bulk copies of the tile's inputs (one contiguous block
  // of mt x J values per field) and of the forward basis; TMEM; coefficients; blow-up gate
  if (threadIdx.x == 0) {
    *sflag = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) tc::mbar_init(&mbar[q], 1);
    tc::fence_mbar_init();
    const uint32_t row_bytes = (uint32_t)(mt * J * sizeof(T2));
    tc::mbar_expect_tx(&mbar[3], row_bytes * TC_NIN);
#pragma unroll
    for (int q = 0; q < TC_NIN; ++q) {
      const int f = stage_field(q);
      tc::bulk_g2s(sA + (size_t)q * TC_MT * J * 2, G.four + (size_t)f * FS + ((size_t)m * G.B + b0) * J, row_bytes,
                   &mbar[3]);
    }
    n_in = 1;
    tc::mbar_expect_tx(&mbar[0], (uint32_t)(TC_B1 * sizeof(float)));
    tc::bulk_g2s(sB, gbasis + (size_t)m * TC_BLOCK, (uint32_t)(TC_B1 * sizeof(float)), &mbar[0]);
    n_tma = 1;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, TC_TMEM_COLS);
    tc::tmem_relinquish();
  }
  load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, TC_MT, cnt, TC_CNT, sig, sigP, sigm1, sigPm1, tcmn);
  if (threadIdx.x < TC_MT) {
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

  // ---- phase 1: combined, symmetrised inputs of (member, j') from the staged
  // copy; a warp covers 4 members x 8 j'
  const int jp = (warp & 3) * 8 + (lane & 7);
  const int bt = (warp >> 2) * 4 + (lane >> 3);
  T2 xs[NSLOT], xa[NSLOT];
  // the combination's step factors at (member, j') and its mirror latitude,
  // loaded while the input copies are in flight
  StepCoefs<T> kc0{}, kc1{};
  if (bt < mt) {
    kc0 = load_step_coefs<T>(G, b0 + bt, jp);
    kc1 = kc0;
    kc1.tsc = G.jco[(size_t)(b0 + bt) * J + (J - 1 - jp)];
  }
  // write-out: thread -> member wbt, latitudes wj, wj + 1 (16-byte accesses)
  static_assert(TC_MT * TC_J == 2 * 256, "one latitude pair per thread");
  const int wbt = threadIdx.x / (TC_J / 2), wj = 2 * (threadIdx.x % (TC_J / 2));
  T2 pold[3][2], pmid[3][2];  // its carries, loaded ahead of GEMM2
  T wal = (T)0, wan = (T)0;   // its filter weights, loaded with them
  // one thread waits on each mbarrier and the block barrier releases the rest:
  // 256 spinning threads would take issue slots from the co-resident CTA
  bool ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[3], 0, basis.wait_limit) : true;
  ok = __syncthreads_and(ok);
  if (ok) {
    const T2* stg = (const T2*)sA;
    if (bt < mt) {
      const int b = b0 + bt;
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int j = side ? (J - 1 - jp) : jp;
        T2 c[NSLOT];
        step_combos_ld<T>(G, cfg, 0, incr, m, b, j,
                          [&](int f) { return stg[(stage_slot(f) * TC_MT + bt) * J + j]; }, c, side ? &kc1 : &kc0);
        if (side == 0) {
#pragma unroll
          for (int q = 0; q < NSLOT; ++q) { xs[q] = c[q]; xa[q] = c[q]; }
        } else {
#pragma unroll
          for (int q = 0; q < NSLOT; ++q) { xs[q] = cadd(xs[q], c[q]); xa[q] = csub(xa[q], c[q]); }
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) { xs[q] = mk<T2>(0, 0); xa[q] = xs[q]; }
    }
  }
  // parity 0: P slots take the symmetric sum and H slots the antisymmetric one; parity 1 the reverse
  auto write_A1 = [&](int par) {
    float* aH = sA;
    float* aL = sA + TC_ROWS * TC_K1;
#pragma unroll
    for (int gq = 0; gq < 8; ++gq) {
      const int sp = group_p(gq), sh = group_h(gq);
      const T2 vp = par ? xa[sp] : xs[sp];
      T2 vh = mk<T2>(0, 0);
      if (sh >= 0) vh = par ? xs[NSPX + sh] : xa[NSPX + sh];
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        const int row = gq * 16 + bt * 2 + comp;
        float hi, lo;
        tc::split_tf32(comp ? vp.y : vp.x, hi, lo);
        aH[tc::cm_index(row, jp, TC_K1)] = hi;
        aL[tc::cm_index(row, jp, TC_K1)] = lo;
        tc::split_tf32(comp ? vh.y : vh.x, hi, lo);
        aH[tc::cm_index(row, TC_JH + jp, TC_K1)] = hi;
        aL[tc::cm_index(row, TC_JH + jp, TC_K1)] = lo;
      }
    }
  };
  const uint32_t idesc1 = tc::idesc_tf32(TC_ROWS, TC_N1), idesc1w = tc::idesc_tf32(TC_ROWS, 2 * TC_N1);
  const uint32_t idesc2 = tc::idesc_tf32(TC_ROWS, TC_N2);
  const uint32_t aHs = tc::smem_u32(sA), aLs = aHs + (uint32_t)(TC_ROWS * TC_K1 * 4);
  const uint32_t bbase = tc::smem_u32(sB);

  // ---- phase 2: GEMM1, parity 0 then parity 1 (the A buffer is refilled in between)
  if (ok) {
    __syncthreads();  // every thread has read its staged inputs: A1 overwrites them
    write_A1(0);
    tc::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (!tc::mbar_wait_bounded(&mbar[0], 0, basis.wait_limit)) *sflag = 1;
      if (!*sflag) mma_3xtf32_2(tbase, aHs, aLs, bbase, TC_N1, TC_K1, idesc1w, idesc1);
      tc::mma_commit(&mbar[1]);
      n_c1 = 1;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;  // written by thread 0 before the barrier: the same value for every thread
  }
  if (ok) {
    write_A1(1);
    tc::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t b1 = bbase + 2u * TC_N1 * TC_K1 * 4u;
      mma_3xtf32_2(tbase + 2 * TC_N1, aHs, aLs, b1, TC_N1, TC_K1, idesc1w, idesc1);
      tc::mma_commit(&mbar[1]);
      n_c1 = 2;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 1, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
  }
  if (ok) {
    // B1 is no longer read: fetch B2 into the same buffer, overlapped with the epilogue
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(&mbar[0], (uint32_t)(TC_B2 * sizeof(float)));
      tc::bulk_g2s(sB, gbasis + (size_t)m * TC_BLOCK + TC_B1, (uint32_t)(TC_B2 * sizeof(float)), &mbar[0]);
      n_tma = 2;
    }
    // ---- phase 3: D1 -> staging sRes[g][n-m][member, re/im]; zero the A2 operands
    {
      const int quarter = warp & 3, par = warp >> 2;
      const int row = quarter * 32 + lane;
      const int gq = row >> 4, btc = row & 15;
      const int Cp = par ? C1 : C0;
#pragma unroll
      for (int c0 = 0; c0 < TC_N1; c0 += 16) {
        float v[16], v1[16];
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * par * TC_N1 + c0), v);
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((2 * par + 1) * TC_N1 + c0), v1);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += v1[i];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = c0 + i;
          if (c < Cp) sRes[(gq * TC_CNT + (par + 2 * c)) * 16 + btc] = v[i];
        }
      }
    }
    for (int i = threadIdx.x; i < TC_RES0; i += blockDim.x) sA[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 4: spectral epilogue -> A2 operands [par][hi, lo][112 rows][K2]
    for (int t = threadIdx.x; t < TC_MT * cnt; t += blockDim.x) {
      const int bti = t % TC_MT, kk = t / TC_MT, n = m + kk;
      const int par = kk & 1, c = kk >> 1;
      const T s = sig[bti * TC_CNT + kk], sp = sigP[bti * TC_CNT + kk], tcv = tcmn[bti * TC_CNT + kk];
      const T sm1 = sigm1[bti * TC_CNT + kk], spm1 = sigPm1[bti * TC_CNT + kk];
      const T nn1 = (T)(n * (n + 1));
      const T om = bti < mt ? G.mco[MC_OM * G.B + b0 + bti] : (T)0;
      T kv[7][2];
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        auto S = [&](int gq) { return sRes[(gq * TC_CNT + kk) * 16 + bti * 2 + comp]; };
        const T sphi = S(0) + nn1 * S(1);
        const T sdel = S(2) + nn1 * S(3);
        const T seta = S(4);
        T cdel, ceta, kphi, kdel, keta;
        if (incr) {
          // new = curr + Inv(dc), dc = (sigma - 1) Fwd(curr) + sigma * tendency
          const T iphi = S(5), idel = S(6), ieta = S(7);
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
      float* aH = sA + (size_t)(2 * par) * TC_A2;
      float* aL = aH + TC_A2;
#pragma unroll
      for (int q = 0; q < 7; ++q)
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = q * 16 + bti * 2 + comp;
          float hi, lo;
          tc::split_tf32(kv[q][comp], hi, lo);
          aH[tc::cm_index(row, c, TC_K2)] = hi;
          aL[tc::cm_index(row, c, TC_K2)] = lo;
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- phase 5: GEMM2, both parities (rows 112..127 read the staging area and are ignored)
    // Each thread first issues the global loads of its write-out pair, so that
    // their latency overlaps the GEMM.
    if (wbt < mt) {
      load_step_rows<T>(G, cfg, incr, FS, ((size_t)m * G.B + b0 + wbt) * J + wj, pold, pmid);
      wal = G.mco[(cfg.raw ? MC_RAWM : MC_ALPHA) * G.B + b0 + wbt];
      wan = cfg.raw ? G.mco[MC_RAWN * G.B + b0 + wbt] : (T)0;
    }
    if (threadIdx.x == 0) {
      if (!tc::mbar_wait_bounded(&mbar[0], 1, basis.wait_limit)) *sflag = 1;
      if (!*sflag) {
        for (int par = 0; par < 2; ++par) {
          const uint32_t a2 = aHs + (uint32_t)(2 * par * TC_A2) * 4u;
          const uint32_t bp = bbase + (uint32_t)(2 * par * TC_N2 * TC_K2) * 4u;
          mma_3xtf32(tbase + 2 * TC_N1 + par * TC_N2, a2, a2 + TC_A2 * 4, bp, bp + TC_N2 * TC_K2 * 4, TC_K2,
                     idesc2);
        }
      }
      tc::mma_commit(&mbar[2]);
      n_c2 = 1;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[2], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;
  }
  if (ok) {
    // ---- phase 6: D2 -> output staging Out[f][member][j][re/im]; f 0..4 from the P
    // columns of rows q 0..4, f 5, 6 from the H columns of rows q 5, 6
    float* Out = sA;
    {
      const int quarter = warp & 3, half = warp >> 2;
      const int row = quarter * 32 + lane;
      const int q = row >> 4, btc = row & 15, bti = btc >> 1, comp = btc & 1;
      const bool hcols = half == 1;
      const bool active = hcols ? (q == 5 || q == 6) : (q <= 4);
      const uint32_t lanes = (uint32_t)(quarter * 32) << 16;
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const int col0 = half * TC_JH + cc * 16;
        float E[16], O[16];
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * TC_N1 + col0), E);
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * TC_N1 + TC_N2 + col0), O);
        if (active) {
          float* o = Out + (size_t)(q * TC_MT + bti) * TC_OST + comp;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int jj = cc * 16 + i;
            o[2 * jj] = E[i] + O[i];
            o[2 * (J - 1 - jj)] = hcols ? (O[i] - E[i]) : (E[i] - O[i]);
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 7: write-out and carries, by latitude pairs (16-byte accesses, coalesced along j)
    if (wbt < mt && !sdead[wbt]) {
      const size_t o = ((size_t)m * G.B + b0 + wbt) * J + wj;
      auto get = [&](int f, int e) { return *(const float2*)&Out[(size_t)(f * TC_MT + wbt) * TC_OST + 2 * (wj + e)]; };
      T2 nw[3][2], uu[2], vv[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        nw[0][e] = get(0, e);
        nw[1][e] = get(1, e);
        nw[2][e] = get(2, e);
        uu[e] = cadd(get(3, e), get(5, e));
        vv[e] = cadd(get(4, e), get(6, e));
      }
      store_step_rows<T>(G, cfg, incr, FS, o, wal, wan, nw, cfg.test != 1, uu, vv, pold, pmid);
    }
    if (m == 0 && threadIdx.x < mt && !sdead[threadIdx.x]) {
      const int b = b0 + threadIdx.x;
      double wc = G.member[MS_WCURR * G.B + b], wm = G.member[MS_WMID * G.B + b];
      step_residual_weights(cfg, G.par[P_ALPHA * G.B + b], G.par[P_WALPHA * G.B + b], wc, wm);
      G.member[MS_WMID * G.B + b] = wm;
      G.member[MS_WCURR * G.B + b] = wc;
      G.member[MS_UPDATED * G.B + b] = 1.0;
    }
  } else {
    // a wait ran out: report, then drain (bounded) what this CTA issued before freeing TMEM
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      if (n_in > 0) tc::mbar_wait_bounded(&mbar[3], 0, 1u << 20);
      if (n_tma > 0) tc::mbar_wait_bounded(&mbar[0], (uint32_t)(n_tma - 1), 1u << 20);
      if (n_c1 > 0) tc::mbar_wait_bounded(&mbar[1], (uint32_t)(n_c1 - 1), 1u << 20);
      if (n_c2 > 0) tc::mbar_wait_bounded(&mbar[2], 0, 1u << 20);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, TC_TMEM_COLS);
}


// ===========================================================================
// Adjoint of k_spectral_tc (modified Euler), the tensor-core form of
// k_spectral_adj (spectral.cu):
//   GEMM1' (transposed inverse Legendre), per parity:
//     D1'[row, c] = sum_k A1'[row, k] B1'[c, k]
//     row = group q (7: lambda of eta, delta, Phi, Uprep, Vprep on P; of U, V on
//     H) x member x re/im = 112 of 128 rows, k = [P at j' | H at j'] (unweighted)
//   epilogue: transposed wind inversion, n(n+1), hyperdiffusion, incremental form
//   GEMM2' (transposed forward Legendre), per parity:
//     D2'[row, col] = sum_c A2'[row, c] B2'[col, c]
//     row = slot q (8: PhiP1, PhiP2, dP1, dP2, eP1, identity Phi, delta, eta)
//     x member x re/im = 128 rows, col = [Pw at j' | Hw at j']; the Hw columns
//     of slots 0, 2, 3, 4 are the H slots PhiH1, dH1, dH2, eH1
//   write-out: adj_store_rows (transposed combination) + Phibar gradient.
// ===========================================================================
namespace {
constexpr int TCA_NIN = 5;                          // staged lambda of eta, delta, Phi, U, V
constexpr int TCA_A2 = TC_ROWS * TC_K2;             // one A2' operand: 128 rows (3072 floats)
constexpr int TCA_RES0 = 4 * TCA_A2;                // D1' staging after the A2' operands
constexpr int TCA_RES = 7 * TC_CNT * 16;            // [q][n-m][member, re/im]
constexpr int TCA_NOUT = 12;                        // 8 P slots + 4 H slots
constexpr int TCA_A = TCA_RES0 + TCA_RES > TC_A ? TCA_RES0 + TCA_RES : TC_A;
static_assert(TCA_NOUT * TC_MT * TC_OST <= TCA_A, "adjoint output staging must fit in the A region");
static_assert(TCA_NIN * TC_MT * TC_J * 2 <= TCA_A, "staged lambda must fit in the A region");
__host__ __device__ constexpr int adj_hslot(int q) {  // H result of GEMM2' row group q, or -1
  return q == 0 ? 0 : q == 2 ? 1 : q == 3 ? 2 : q == 4 ? 3 : -1;
}
}  // namespace

size_t spec_tc_adj_smem_bytes() { return (size_t)(TCA_A + TC_B1 + TC_COEF) * sizeof(float) + 256; }

__global__ void __launch_bounds__(256, 2) k_spectral_adj_tc(const __grid_constant__ SpecLaunch<float> L,
                                                            const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NKADJ = 8;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const float* gbasis = basis.p[gi];
  const StepCfg& cfg = L.cfg;
  const int J = TC_J;
  const int m = idx / G.ntb;
  const int b0 = (idx % G.ntb) * TC_MT;
  const int mt = min(TC_MT, G.B - b0);
  const int cnt = TC_CNT - m, C0 = (cnt + 1) / 2, C1 = cnt / 2;
  const size_t FS = (size_t)TC_CNT * G.B * J;
  const bool incr = cfg.incremental != 0;
  if (cfg.scheme != 0) {  // the host launches this kernel for modified-Euler steps only
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }

  float* sA = (float*)smem_raw;            // staged lambda | A1' | A2' + D1' staging | output staging
  float* sB = sA + TCA_A;                  // B1', then B2'
  float* sRes = sA + TCA_RES0;
  float* sig = sB + TC_B1;
  float* sigP = sig + TC_MT * TC_CNT;
  float* sigm1 = sigP + TC_MT * TC_CNT;
  float* sigPm1 = sigm1 + TC_MT * TC_CNT;
  float* tcmn = sigPm1 + TC_MT * TC_CNT;
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + TC_MT * TC_CNT) + 15) & ~(uintptr_t)15);  // [4]
  uint32_t* tslot = (uint32_t*)(mbar + 4);
  int* sflag = (int*)(tslot + 1);
  double* sgrad = (double*)(((uintptr_t)(sflag + 1) + 15) & ~(uintptr_t)15);  // [MT][2]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int n_tma = 0, n_in = 0, n_c1 = 0, n_c2 = 0;

  // ---- phase 0: barriers; bulk copies of lambda_Y (5 fields) and of B1'; TMEM; coefficients
  if (threadIdx.x == 0) {
    *sflag = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) tc::mbar_init(&mbar[q], 1);
    tc::fence_mbar_init();
    const uint32_t row_bytes = (uint32_t)(mt * J * sizeof(T2));
    tc::mbar_expect_tx(&mbar[3], row_bytes * TCA_NIN);
#pragma unroll
    for (int q = 0; q < TCA_NIN; ++q)
      tc::bulk_g2s(sA + (size_t)q * TC_MT * J * 2, G.lamY + (size_t)q * FS + ((size_t)m * G.B + b0) * J, row_bytes,
                   &mbar[3]);
    n_in = 1;
    tc::mbar_expect_tx(&mbar[0], (uint32_t)(TC_B1 * sizeof(float)));
    tc::bulk_g2s(sB, gbasis + (size_t)m * TC_BLOCK, (uint32_t)(TC_B1 * sizeof(float)), &mbar[0]);
    n_tma = 1;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, TC_TMEM_COLS);
    tc::tmem_relinquish();
  }
  load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, TC_MT, cnt, TC_CNT, sig, sigP, sigm1, sigPm1, tcmn);
  if (threadIdx.x < 2 * TC_MT) sgrad[threadIdx.x] = 0.0;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  // ---- phase 1: symmetrised lambda_Y of (member, j')
  const int jp = (warp & 3) * 8 + (lane & 7);
  const int bt = (warp >> 2) * 4 + (lane >> 3);
  T2 ys[TCA_NIN], ya[TCA_NIN];
  // write-out: warp -> member, lane -> latitudes 2 lane, 2 lane + 1 (16-byte accesses)
  static_assert(TC_MT * TC_J == 2 * 256 && TC_J == 64, "one latitude pair per thread, a member per warp");
  const int wbt = warp, wj = 2 * lane;
  AdjRowsIn<T> pin;  // its inputs, loaded ahead of GEMM2'
  bool ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[3], 0, basis.wait_limit) : true;
  ok = __syncthreads_and(ok);
  if (ok) {
    const T2* stg = (const T2*)sA;
#pragma unroll
    for (int f = 0; f < TCA_NIN; ++f) {
      if (bt < mt) {
        const T2 u = stg[(f * TC_MT + bt) * J + jp], v = stg[(f * TC_MT + bt) * J + (J - 1 - jp)];
        ys[f] = cadd(u, v);
        ya[f] = csub(u, v);
      } else {
        ys[f] = mk<T2>(0, 0);
        ya[f] = ys[f];
      }
    }
  }
  // parity 0: the P groups take the symmetric sums, the H groups the antisymmetric ones
  auto write_A1 = [&](int par) {
    float* aH = sA;
    float* aL = sA + TC_ROWS * TC_K1;
#pragma unroll
    for (int gq = 0; gq < 7; ++gq) {
      const bool hg = gq >= 5;
      const int f = hg ? gq - 2 : gq;  // H groups carry lambda U, V
      const T2 v = hg ? (par ? ys[f] : ya[f]) : (par ? ya[f] : ys[f]);
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        const int row = gq * 16 + bt * 2 + comp;
        float hi, lo;
        tc::split_tf32(comp ? v.y : v.x, hi, lo);
        aH[tc::cm_index(row, hg ? TC_JH + jp : jp, TC_K1)] = hi;
        aL[tc::cm_index(row, hg ? TC_JH + jp : jp, TC_K1)] = lo;
        aH[tc::cm_index(row, hg ? jp : TC_JH + jp, TC_K1)] = 0.f;
        aL[tc::cm_index(row, hg ? jp : TC_JH + jp, TC_K1)] = 0.f;
      }
    }
  };
  const uint32_t idesc1 = tc::idesc_tf32(TC_ROWS, TC_N1), idesc1w = tc::idesc_tf32(TC_ROWS, 2 * TC_N1);
  const uint32_t idesc2 = tc::idesc_tf32(TC_ROWS, TC_N2);
  const uint32_t aHs = tc::smem_u32(sA), aLs = aHs + (uint32_t)(TC_ROWS * TC_K1 * 4);
  const uint32_t bbase = tc::smem_u32(sB);

  // ---- phase 2: GEMM1', parity 0 then parity 1
  if (ok) {
    __syncthreads();  // the staged lambda is read: A1' overwrites it
    write_A1(0);
    tc::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (!tc::mbar_wait_bounded(&mbar[0], 0, basis.wait_limit)) *sflag = 1;
      if (!*sflag) mma_3xtf32_2(tbase, aHs, aLs, bbase, TC_N1, TC_K1, idesc1w, idesc1);
      tc::mma_commit(&mbar[1]);
      n_c1 = 1;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;
  }
  if (ok) {
    write_A1(1);
    tc::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t b1 = bbase + 2u * TC_N1 * TC_K1 * 4u;
      mma_3xtf32_2(tbase + 2 * TC_N1, aHs, aLs, b1, TC_N1, TC_K1, idesc1w, idesc1);
      tc::mma_commit(&mbar[1]);
      n_c1 = 2;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 1, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
  }
  if (ok) {
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(&mbar[0], (uint32_t)(TC_B2 * sizeof(float)));
      tc::bulk_g2s(sB, gbasis + (size_t)m * TC_BLOCK + TC_B1, (uint32_t)(TC_B2 * sizeof(float)), &mbar[0]);
      n_tma = 2;
    }
    // ---- phase 3: D1' -> sRes[q][n-m][member, re/im]; zero the A2' operands
    {
      const int quarter = warp & 3, par = warp >> 2;
      const int row = quarter * 32 + lane;
      const int gq = row >> 4, btc = row & 15;
      const int Cp = par ? C1 : C0;
#pragma unroll
      for (int c0 = 0; c0 < TC_N1; c0 += 16) {
        float v[16], v1[16];
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * par * TC_N1 + c0), v);
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((2 * par + 1) * TC_N1 + c0), v1);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += v1[i];
        if (gq < 7) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int c = c0 + i;
            if (c < Cp) sRes[(gq * TC_CNT + (par + 2 * c)) * 16 + btc] = v[i];
          }
        }
      }
    }
    for (int i = threadIdx.x; i < TCA_RES0; i += blockDim.x) sA[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 4: transposed wind inversion, n(n+1), hyperdiffusion -> A2' [par][hi, lo][128][K2]
    for (int t = threadIdx.x; t < TC_MT * cnt; t += blockDim.x) {
      const int bti = t % TC_MT, kk = t / TC_MT, n = m + kk;
      const int par = kk & 1, c = kk >> 1;
      auto S = [&](int q, int comp) { return sRes[(q * TC_CNT + kk) * 16 + bti * 2 + comp]; };
      const T xm = (T)m;
      const T tcv = tcmn[bti * TC_CNT + kk];
      const T s = sig[bti * TC_CNT + kk], sp = sigP[bti * TC_CNT + kk];
      const T sm1 = sigm1[bti * TC_CNT + kk], spm1 = sigPm1[bti * TC_CNT + kk];
      const T nn1 = (T)(n * (n + 1));
      // lambda delta_s = (i m) lambda Uprep - lambda Hin_V ; lambda eta_s = (i m) lambda Vprep + lambda Hin_U
      const T lds_r = -xm * S(3, 1) - S(6, 0), lds_i = xm * S(3, 0) - S(6, 1);
      const T les_r = -xm * S(4, 1) + S(5, 0), les_i = xm * S(4, 0) + S(5, 1);
      const T w = (n == 0) ? (T)0 : tcv;
      const T lce_r = S(0, 0) + w * les_r, lce_i = S(0, 1) + w * les_i;
      const T lcd_r = S(1, 0) + w * lds_r, lcd_i = S(1, 1) + w * lds_i;
      const T lcp_r = S(2, 0), lcp_i = S(2, 1);
      T kv[NKADJ][2];
      kv[0][0] = sp * lcp_r; kv[0][1] = sp * lcp_i;
      kv[1][0] = nn1 * sp * lcp_r; kv[1][1] = nn1 * sp * lcp_i;
      kv[2][0] = s * lcd_r; kv[2][1] = s * lcd_i;
      kv[3][0] = nn1 * s * lcd_r; kv[3][1] = nn1 * s * lcd_i;
      kv[4][0] = s * lce_r; kv[4][1] = s * lce_i;
      kv[5][0] = incr ? spm1 * S(2, 0) : (T)0; kv[5][1] = incr ? spm1 * S(2, 1) : (T)0;
      kv[6][0] = incr ? (s * w * lds_r + sm1 * S(1, 0)) : (T)0; kv[6][1] = incr ? (s * w * lds_i + sm1 * S(1, 1)) : (T)0;
      kv[7][0] = incr ? (s * w * les_r + sm1 * S(0, 0)) : (T)0; kv[7][1] = incr ? (s * w * les_i + sm1 * S(0, 1)) : (T)0;
      float* aH = sA + (size_t)(2 * par) * TCA_A2;
      float* aL = aH + TCA_A2;
#pragma unroll
      for (int q = 0; q < NKADJ; ++q)
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = q * 16 + bti * 2 + comp;
          float hi, lo;
          tc::split_tf32(kv[q][comp], hi, lo);
          aH[tc::cm_index(row, c, TC_K2)] = hi;
          aL[tc::cm_index(row, c, TC_K2)] = lo;
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- phase 5: GEMM2', both parities; write-out inputs loaded meanwhile
    if (wbt < mt) adj_load_rows<T>(G, incr, FS, ((size_t)m * G.B + b0 + wbt) * J + wj, pin);
    if (threadIdx.x == 0) {
      if (!tc::mbar_wait_bounded(&mbar[0], 1, basis.wait_limit)) *sflag = 1;
      if (!*sflag) {
        for (int par = 0; par < 2; ++par) {
          const uint32_t a2 = aHs + (uint32_t)(2 * par * TCA_A2) * 4u;
          const uint32_t bp = bbase + (uint32_t)(2 * par * TC_N2 * TC_K2) * 4u;
          mma_3xtf32(tbase + 2 * TC_N1 + par * TC_N2, a2, a2 + TCA_A2 * 4, bp, bp + TC_N2 * TC_K2 * 4, TC_K2,
                     idesc2);
        }
      }
      tc::mma_commit(&mbar[2]);
      n_c2 = 1;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[2], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;
  }
  if (ok) {
    // ---- phase 6: D2' -> output staging Out[slot][member][j][re/im]: slots 0..7
    // from the Pw columns of rows q, slots 8..11 from the Hw columns of rows 0, 2, 3, 4
    float* Out = sA;
    {
      const int quarter = warp & 3, half = warp >> 2;
      const int row = quarter * 32 + lane;
      const int q = row >> 4, btc = row & 15, bti = btc >> 1, comp = btc & 1;
      const bool hcols = half == 1;
      const int slot = hcols ? (adj_hslot(q) >= 0 ? NKADJ + adj_hslot(q) : -1) : q;
      const uint32_t lanes = (uint32_t)(quarter * 32) << 16;
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const int col0 = half * TC_JH + cc * 16;
        float E[16], O[16];
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * TC_N1 + col0), E);
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * TC_N1 + TC_N2 + col0), O);
        if (slot >= 0) {
          float* o = Out + (size_t)(slot * TC_MT + bti) * TC_OST + comp;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int jj = cc * 16 + i;
            o[2 * jj] = E[i] + O[i];
            o[2 * (J - 1 - jj)] = hcols ? (O[i] - E[i]) : (E[i] - O[i]);
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 7: transposed combination -> lambda of the state fields; Phibar gradient
    if (wbt < mt) {  // uniform over a warp
      const int b = b0 + wbt;
      const size_t o = ((size_t)m * G.B + b) * J + wj;
      auto ld = [&](int q, int e) { return *(const float2*)&Out[(size_t)(q * TC_MT + wbt) * TC_OST + 2 * (wj + e)]; };
      T gp = adj_store_rows<T, NKADJ>(G, cfg, incr, FS, o, m, b, wj, ld, pin);
      if (G.grad) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) gp += __shfl_xor_sync(0xffffffffu, gp, off);
        if (lane == 0) { sgrad[wbt * 2] = (double)gp; sgrad[wbt * 2 + 1] = 0.0; }
      }
    }
    __syncthreads();
    if (G.grad && threadIdx.x < mt)
      atomicAdd(&G.grad[G_PHIBAR * G.B + b0 + threadIdx.x], sgrad[threadIdx.x * 2] + sgrad[threadIdx.x * 2 + 1]);
  } else {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      if (n_in > 0) tc::mbar_wait_bounded(&mbar[3], 0, 1u << 20);
      if (n_tma > 0) tc::mbar_wait_bounded(&mbar[0], (uint32_t)(n_tma - 1), 1u << 20);
      if (n_c1 > 0) tc::mbar_wait_bounded(&mbar[1], (uint32_t)(n_c1 - 1), 1u << 20);
      if (n_c2 > 0) tc::mbar_wait_bounded(&mbar[2], 0, 1u << 20);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, TC_TMEM_COLS);
}

void spec_tc_set_attributes() {
  cudaFuncSetAttribute(k_spectral_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_tc_smem_bytes());
  cudaFuncSetAttribute(k_spectral_adj_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_tc_adj_smem_bytes());
}

cudaError_t launch_spec_tc(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err, cudaStream_t s) {
  k_spectral_tc<<<nblocks, 256, spec_tc_smem_bytes(), s>>>(L, basis, err);
  return cudaGetLastError();
}

cudaError_t launch_spec_adj_tc(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                               cudaStream_t s) {
  k_spectral_adj_tc<<<nblocks, 256, spec_tc_adj_smem_bytes(), s>>>(L, basis, err);
  return cudaGetLastError();
}

}  // namespace swp
