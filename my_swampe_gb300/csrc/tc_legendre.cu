// Tensor-core (tcgen05) Legendre sandwich of one modified-Euler step, FP32
// fast path, compiled per truncation: M = 42 (64 x 128 Gauss grid, two CTAs
// per SM) and M = 63 (96 x 192, one CTA per SM); M = 106, whose operands do not
// fit in one CTA's shared memory, has its own chunked kernel (tc_legendre106.cu).  The shapes below are those
// of M = 42; TcShape<M, J> gives them for any truncation whose operands fit in
// shared memory.
//
// Same per-m decomposition and arithmetic as k_spectral (spectral.cu), with the
// two contractions issued as kind::tf32 MMAs in 3xTF32 split precision
// (a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accumulation in TMEM):
//   GEMM1, forward Legendre, once per parity of n - m:
//     D1[row, c] = sum_k A1[row, k] B1[c, k]
//     row = group g (8) x member (8) x re/im (2) = 128,
//     k = [Pw at j' (J/2) | Hw at j' (J/2)], c -> n = m + par + 2c (N = 32)
//   epilogue in shared memory: n(n+1), hyperdiffusion, the incremental form,
//     wind-inversion inputs (spectral_transform.py:577-594, filters.py:95-151)
//   GEMM2, inverse Legendre, once per parity:
//     D2[row, col] = sum_c A2[row, c] B2[col, c]
//     row = input q (7) x member (8) x re/im (2) = 112 (of the 128 MMA rows),
//     col = [P at j' (J/2) | H at j' (J/2)]
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
// Operand shapes of truncation M on J Gauss latitudes.
template <int M_, int J_>
struct TcShape {
  static constexpr int M = M_, J = J_, JH = J_ / 2;
  static constexpr int MT = 8;                         // members per CTA
  static constexpr int CNT = M + 1;                    // n = m..M
  static constexpr int HALF = (CNT + 1) / 2;           // n of one parity, at most
  static constexpr int ROWS = 128;                     // MMA M
  static constexpr int K1 = 2 * JH;
  static constexpr int N1 = (HALF + 15) / 16 * 16;     // multiple of 16
  static constexpr int R2 = 112;                       // used rows of GEMM2
  static constexpr int K2 = (HALF + 7) / 8 * 8;        // multiple of 8
  static constexpr int N2 = 2 * JH;
  static constexpr int B1 = 4 * N1 * K1;               // [par][hi, lo][N1][K1]
  static constexpr int B2 = 4 * N2 * K2;               // [par][hi, lo][N2][K2]
  static constexpr int BLOCK = B1 + B2;                // packed basis floats per m
  static constexpr int A = 2 * ROWS * K1;              // A region
  static constexpr int A2 = R2 * K2;                   // one A2 operand
  static constexpr int RES0 = 4 * A2;                  // D1 staging inside the A region
  static constexpr int RES = 8 * CNT * 16;             // [g][n-m][member, re/im]
  static constexpr int OST = 2 * J + 2;                // output staging row stride (floats)
  static constexpr int NOUT = 7;                       // eta, delta, Phi, Uprep, Vprep | U_H, V_H
  static constexpr int COEF = 5 * MT * CNT;
  static constexpr int TMEM_COLS = 256;                // D1: 2 x (2 x N1), D2: 2 x N2 (reusing D1's columns)
  static constexpr int NIN = 11;                       // staged inputs of a modified-Euler step
  // (member, j') pairs of the combination: warp tasks of 4 members x 8 j'
  static constexpr int NTASK = (MT / 4) * (JH / 8);
  static constexpr int NPAIR = (NTASK + 7) / 8;        // per thread
  // write-out latitude pairs (16-byte accesses) per thread
  static constexpr int NWPAIR = (MT * J / 2 + 255) / 256;
  // adjoint
  static constexpr int ANIN = 5;                       // staged lambda of eta, delta, Phi, U, V
  static constexpr int AA2 = ROWS * K2;                // one A2' operand: 128 rows
  static constexpr int ARES0 = 4 * AA2;
  static constexpr int ARES = 7 * CNT * 16;
  static constexpr int ANOUT = 12;                     // 8 P slots + 4 H slots
  static constexpr int AA = ARES0 + ARES > A ? ARES0 + ARES : A;
  static constexpr int MINB = 2 * (A + B1 + COEF) * 4 + 512 <= 227 * 1024 ? 2 : 1;  // CTAs per SM

  static_assert(JH % 16 == 0 && MT % 4 == 0, "latitude blocks of 16, member blocks of 4");
  static_assert(RES0 + RES <= A, "D1 staging must fit in the A region");
  static_assert(NOUT * MT * OST <= A, "output staging must fit in the A region");
  // the MMA reads all 128 rows of the last A2 operand: they must stay in the A region
  static_assert(3 * A2 + ROWS * K2 <= A, "A2 over-read must stay in the A region");
  static_assert(B2 <= B1, "B2 reuses the B1 buffer");
  static_assert(NIN * MT * J * 2 <= A, "staged inputs must fit in the A region");
  static_assert(4 * N1 <= TMEM_COLS && 2 * N1 + 2 * N2 <= TMEM_COLS, "TMEM columns");
  static_assert(N1 <= 128 && N2 <= 256 && N2 % 16 == 0, "MMA N");
  // the hi tile of a [hi, lo][N][K] operand pair is followed by its lo tile at (N / 8) stride offsets
  static_assert(N1 * K1 * 4 == (N1 / 8) * (K1 / 4) * 128, "B1 lo tile must follow its hi tile");
  static_assert(ANOUT * MT * OST <= AA, "adjoint output staging must fit in the A region");
  static_assert(ANIN * MT * J * 2 <= AA, "staged lambda must fit in the A region");
  static_assert(MT * J / 2 <= B1, "the adjoint's Phibar terms reuse the B buffer");
  static_assert(MT <= 8, "one warp per member reduces the adjoint's Phibar terms");
};
typedef TcShape<42, 64> Tc42;
typedef TcShape<63, 96> Tc63;

__host__ __device__ constexpr int stage_field(int q) {  // staged slot -> Fourier field
  return q == 0 ? F_ETA : q == 1 ? F_DELTA : q == 2 ? F_PHI : F_A + (q - 3);
}
// Fourier field -> staged slot, for the fields stage_field covers (F_A..F_G are
// consecutive); any other field is never read by the modified-Euler combination
__host__ __device__ constexpr int stage_slot(int f) {
  return f == F_ETA ? 0 : f == F_DELTA ? 1 : f == F_PHI ? 2 : (f >= F_A && f <= F_G) ? f - F_A + 3 : 0;
}
static_assert(F_G - F_A + 4 == 11, "staged fields");

// slots of forward group g (compile-time, so that the slot arrays stay in registers)
__host__ __device__ constexpr int group_p(int g) {
  return g == 0 ? SP_PHI1 : g == 1 ? SP_PHI2 : g == 2 ? SP_D1 : g == 3 ? SP_D2 : g == 4 ? SP_E1
       : g == 5 ? SP_IPHI : g == 6 ? SP_ID : SP_IE;
}
__host__ __device__ constexpr int group_h(int g) {
  return g == 0 ? SH_PHI1 : g == 2 ? SH_D1 : g == 3 ? SH_D2 : g == 4 ? SH_E1 : -1;
}

template <typename F>
auto tc_dispatch(int M, F f) -> decltype(f(Tc42())) {
  return M == 63 ? f(Tc63()) : f(Tc42());
}
}  // namespace

size_t spec_tc_smem_bytes(int M) {
  if (M == 106) return spec_tc106_smem_bytes();
  return tc_dispatch(M, [](auto S) { return (size_t)(S.A + S.B1 + S.COEF) * sizeof(float) + 256; });
}
size_t spec_tc_basis_floats(int M) {
  if (M == 106) return spec_tc106_basis_floats();
  return tc_dispatch(M, [](auto S) { return (size_t)S.CNT * S.BLOCK; });
}
size_t spec_tc_adj_basis_floats(int M) { return spec_tc_basis_floats(M); }
int spec_tc_members_per_cta() { return 8; }
bool spec_tc_supported(int M) { return M == 42 || M == 63 || M == 106; }
bool spec_tc_adj_supported(int M) { return spec_tc_supported(M); }

// Pack the FP64 basis into the per-m GEMM operand blocks of shape S.
template <class S>
__global__ void k_pack_tc_basis(const double* __restrict__ Pw_f, const double* __restrict__ Hw_f,
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
    float* b1h = blk + (size_t)(2 * par) * S::N1 * S::K1;
    float* b1l = b1h + S::N1 * S::K1;
    float* b2h = blk + S::B1 + (size_t)(2 * par) * S::N2 * S::K2;
    float* b2l = b2h + S::N2 * S::K2;
    for (int i = threadIdx.x; i < Cp * S::K1; i += blockDim.x) {
      const int c = i / S::K1, k = i % S::K1, jp = k % S::JH;
      const double v = (k < S::JH) ? Pw_f[base + poff + jp * Cp + c] : Hw_f[base + poff + jp * Cp + c];
      const float hi = tc::to_tf32((float)v);
      b1h[tc::cm_index(c, k, S::K1)] = hi;
      b1l[tc::cm_index(c, k, S::K1)] = tc::to_tf32((float)(v - (double)hi));
    }
    for (int i = threadIdx.x; i < S::N2 * Cp; i += blockDim.x) {
      const int col = i / Cp, c = i % Cp, jp = col % S::JH;
      const double v = (col < S::JH) ? P_i[base + poff + c * S::JH + jp] : H_i[base + poff + c * S::JH + jp];
      const float hi = tc::to_tf32((float)v);
      b2h[tc::cm_index(col, c, S::K2)] = hi;
      b2l[tc::cm_index(col, c, S::K2)] = tc::to_tf32((float)(v - (double)hi));
    }
  }
}

namespace {
int pack_basis(const GroupGeom& gg, const double* f1, const double* f2, const double* i1, const double* i2,
               float* out, cudaStream_t s) {
  if (!spec_tc_supported(gg.M)) return SWP_ERR_ARG;
  return tc_dispatch(gg.M, [&](auto S) {
    typedef decltype(S) Sh;
    if (gg.J != Sh::J) return SWP_ERR_ARG;
    k_pack_tc_basis<Sh><<<Sh::CNT, 256, 0, s>>>(f1, f2, i1, i2, gg.boff, out);
    return cudaGetLastError() == cudaSuccess ? SWP_OK : SWP_ERR_CUDA;
  });
}
}  // namespace

int pack_tc_basis(const GroupGeom& gg, float* out, cudaStream_t s) {
  if (gg.M == 106) return pack_tc106_basis(gg, out, false, s);
  return pack_basis(gg, gg.b64[B_PW_F], gg.b64[B_HW_F], gg.b64[B_P_I], gg.b64[B_H_I], out, s);
}

// The adjoint's operand blocks: GEMM1' contracts with the unweighted basis in
// the forward layout (transposed inverse Legendre), GEMM2' with the weighted
// basis in the inverse layout (transposed forward Legendre).
int pack_tc_basis_adj(const GroupGeom& gg, float* out, cudaStream_t s) {
  if (gg.M == 106) return pack_tc106_basis(gg, out, true, s);
  return pack_basis(gg, gg.b64[B_P_F], gg.b64[B_H_F], gg.b64[B_PW_I], gg.b64[B_HW_I], out, s);
}

namespace {
// The MMAs are issued by warp 0 as a whole (warp-collective forms, one elected
// lane issues), with the descriptors of a K-sweep built once and advanced by
// 256 bytes (8 TF32 columns of the core-matrix layout) per K-step.
// the three products of one 3xTF32 K-sweep into d_tmem (K a multiple of 8)
__device__ __forceinline__ void mma_3xtf32(uint32_t d_tmem, uint32_t aH, uint32_t aL, uint32_t bH, uint32_t bL, int K,
                                           uint32_t idesc) {
  const uint32_t sbo = (uint32_t)(K / 4) * 128u;
  const uint64_t dAH = tc::make_desc(aH, 128, sbo), dAL = tc::make_desc(aL, 128, sbo);
  const uint64_t dBH = tc::make_desc(bH, 128, sbo), dBL = tc::make_desc(bL, 128, sbo);
  for (int kk = 0; kk < K / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBH, off), idesc, kk > 0);
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBL, off), idesc, 1);
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAL, off), tc::desc_advance(dBH, off), idesc, 1);
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
  const uint64_t dAH = tc::make_desc(aH, 128, sbo), dAL = tc::make_desc(aL, 128, sbo);
  const uint64_t dBH = tc::make_desc(bH, 128, sbo);
  for (int kk = 0; kk < K / 8; ++kk) {
    const uint32_t off = (uint32_t)kk * 256u;
    tc::mma_tf32_warp(d_tmem, tc::desc_advance(dAH, off), tc::desc_advance(dBH, off), idesc_2n, kk > 0);
    tc::mma_tf32_warp(d_tmem + (uint32_t)n, tc::desc_advance(dAL, off), tc::desc_advance(dBH, off), idesc_n, 1);
  }
}
}  // namespace

template <class S>
__global__ void __launch_bounds__(256, S::MINB) k_spectral_tc(const __grid_constant__ SpecLaunch<float> L,
                                                              const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NSPX = SlotCount<float>::NP;
  constexpr int NSLOT = NSPX + NSH;
  constexpr int MT = S::MT, J = S::J, JH = S::JH, CNT = S::CNT;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  pdl_trigger();
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const float* gbasis = basis.p[gi];
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

  float* sA = (float*)smem_raw;            // staged inputs | A1 | A2 + D1 staging | output staging
  float* sB = sA + S::A;                   // B1, then B2
  float* sRes = sA + S::RES0;
  float* sig = sB + S::B1;                 // [MT][CNT] x 5
  float* sigP = sig + MT * CNT;
  float* sigm1 = sigP + MT * CNT;
  float* sigPm1 = sigm1 + MT * CNT;
  float* tcmn = sigPm1 + MT * CNT;
  // [4]: 0 basis copies, 1 GEMM1 commits, 2 GEMM2 commit, 3 input copies
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + MT * CNT) + 15) & ~(uintptr_t)15);
  uint32_t* tslot = (uint32_t*)(mbar + 4);
  int* sflag = (int*)(tslot + 1);
  int* sdead = sflag + 1;                  // [MT]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // what thread 0 has issued, for the bounded drain on failure
  int n_tma = 0, n_in = 0, n_c1 = 0, n_c2 = 0;

  // ---- phase 0: barriers; bulk copies of the forward basis and of the tile's
  // inputs (one contiguous block of mt x J values per field); TMEM;
  // coefficients; blow-up gate.  The basis and TMEM do not depend on the
  // previous kernel in the stream: they come before the wait for it.
  if (threadIdx.x == 0) {
    *sflag = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) tc::mbar_init(&mbar[q], 1);
    tc::fence_mbar_init();
    tc::mbar_expect_tx(&mbar[0], (uint32_t)(S::B1 * sizeof(float)));
    tc::bulk_g2s(sB, gbasis + (size_t)m * S::BLOCK, (uint32_t)(S::B1 * sizeof(float)), &mbar[0]);
    n_tma = 1;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, S::TMEM_COLS);
    tc::tmem_relinquish();
  }
  pdl_wait();
  if (threadIdx.x == 0) {
    const uint32_t row_bytes = (uint32_t)(mt * J * sizeof(T2));
    tc::mbar_expect_tx(&mbar[3], row_bytes * S::NIN);
#pragma unroll
    for (int q = 0; q < S::NIN; ++q) {
      const int f = stage_field(q);
      tc::bulk_g2s(sA + (size_t)q * MT * J * 2, G.four + (size_t)f * FS + ((size_t)m * G.B + b0) * J, row_bytes,
                   &mbar[3]);
    }
    n_in = 1;
  }
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

  // ---- phase 1: combined, symmetrised inputs of (member, j') from the staged
  // copy.  A warp task covers 4 members x 8 j'; thread k of a task takes member
  // 4 mb + lane / 8 and latitude 8 jb + lane % 8.
  int jp[S::NPAIR], bt[S::NPAIR];
  bool has[S::NPAIR];
#pragma unroll
  for (int k = 0; k < S::NPAIR; ++k) {
    const int task = warp + 8 * k;
    has[k] = task < S::NTASK;
    const int jb = has[k] ? task % (JH / 8) : 0, mb = has[k] ? task / (JH / 8) : 0;
    jp[k] = jb * 8 + (lane & 7);
    bt[k] = mb * 4 + (lane >> 3);
  }
  T2 xs[S::NPAIR][NSLOT], xa[S::NPAIR][NSLOT];
  // the combination's step factors at (member, j') and its mirror latitude,
  // loaded while the input copies are in flight
  StepCoefs<T> kc0[S::NPAIR], kc1[S::NPAIR];
#pragma unroll
  for (int k = 0; k < S::NPAIR; ++k) {
    kc0[k] = StepCoefs<T>{};
    kc1[k] = StepCoefs<T>{};
    if (has[k] && bt[k] < mt) {
      kc0[k] = load_step_coefs<T>(G, b0 + bt[k], jp[k]);
      kc1[k] = kc0[k];
      kc1[k].tsc = G.jco[(size_t)(b0 + bt[k]) * J + (J - 1 - jp[k])];
    }
  }
  // write-out: thread -> member wbt, latitudes wj, wj + 1 (16-byte accesses)
  int wbt[S::NWPAIR], wj[S::NWPAIR];
#pragma unroll
  for (int k = 0; k < S::NWPAIR; ++k) {
    const int q = threadIdx.x + 256 * k;
    wbt[k] = q < MT * J / 2 ? q / (J / 2) : MT;
    wj[k] = 2 * (q % (J / 2));
  }
  T2 pold[S::NWPAIR][3][2], pmid[S::NWPAIR][3][2];  // its carries, loaded ahead of GEMM2
  T wal[S::NWPAIR], wan[S::NWPAIR];                 // its filter weights, loaded with them
  // one thread waits on each mbarrier and the block barrier releases the rest:
  // 256 spinning threads would take issue slots from the co-resident CTA
  bool ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[3], 0, basis.wait_limit) : true;
  ok = __syncthreads_and(ok);
  if (ok) {
    const T2* stg = (const T2*)sA;
#pragma unroll
    for (int k = 0; k < S::NPAIR; ++k) {
      if (has[k] && bt[k] < mt) {
        const int b = b0 + bt[k];
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const int j = side ? (J - 1 - jp[k]) : jp[k];
          T2 c[NSLOT];
          step_combos_ld<T>(G, cfg, 0, incr, m, b, j,
                            [&](int f) { return stg[(stage_slot(f) * MT + bt[k]) * J + j]; }, c,
                            side ? &kc1[k] : &kc0[k]);
          if (side == 0) {
#pragma unroll
            for (int q = 0; q < NSLOT; ++q) { xs[k][q] = c[q]; xa[k][q] = c[q]; }
          } else {
#pragma unroll
            for (int q = 0; q < NSLOT; ++q) { xs[k][q] = cadd(xs[k][q], c[q]); xa[k][q] = csub(xa[k][q], c[q]); }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < NSLOT; ++q) { xs[k][q] = mk<T2>(0, 0); xa[k][q] = xs[k][q]; }
      }
    }
  }
  // parity 0: P slots take the symmetric sum and H slots the antisymmetric one; parity 1 the reverse
  auto write_A1 = [&](int par) {
    float* aH = sA;
    float* aL = sA + S::ROWS * S::K1;
#pragma unroll
    for (int k = 0; k < S::NPAIR; ++k) {
      if (!has[k]) continue;
#pragma unroll
      for (int gq = 0; gq < 8; ++gq) {
        const int sp = group_p(gq), sh = group_h(gq);
        const T2 vp = par ? xa[k][sp] : xs[k][sp];
        T2 vh = mk<T2>(0, 0);
        if (sh >= 0) vh = par ? xs[k][NSPX + sh] : xa[k][NSPX + sh];
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = gq * 16 + bt[k] * 2 + comp;
          float hi, lo;
          tc::split_tf32(comp ? vp.y : vp.x, hi, lo);
          aH[tc::cm_index(row, jp[k], S::K1)] = hi;
          aL[tc::cm_index(row, jp[k], S::K1)] = lo;
          tc::split_tf32(comp ? vh.y : vh.x, hi, lo);
          aH[tc::cm_index(row, JH + jp[k], S::K1)] = hi;
          aL[tc::cm_index(row, JH + jp[k], S::K1)] = lo;
        }
      }
    }
  };
  const uint32_t idesc1 = tc::idesc_tf32(S::ROWS, S::N1), idesc1w = tc::idesc_tf32(S::ROWS, 2 * S::N1);
  const uint32_t idesc2 = tc::idesc_tf32(S::ROWS, S::N2);
  const uint32_t aHs = tc::smem_u32(sA), aLs = aHs + (uint32_t)(S::ROWS * S::K1 * 4);
  const uint32_t bbase = tc::smem_u32(sB);

  // ---- phase 2: GEMM1, parity 0 then parity 1 (the A buffer is refilled in between)
  if (ok) {
    __syncthreads();  // every thread has read its staged inputs: A1 overwrites them
    write_A1(0);
    tc::fence_proxy_async();
    __syncthreads();
    if (warp == 0) {  // warp-collective MMA issue
      const bool good = tc::mbar_wait_bounded_warp(&mbar[0], 0, basis.wait_limit);
      if (!good) *sflag = 1;
      if (good) mma_3xtf32_2(tbase, aHs, aLs, bbase, S::N1, S::K1, idesc1w, idesc1);
      tc::mma_commit_warp(&mbar[1]);
      n_c1 = 1;
    }
    // the epilogue's per-(member, n) coefficients, gathered while the MMAs run
    load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, MT, cnt, CNT, sig, sigP, sigm1, sigPm1, tcmn);
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;  // written by thread 0 before the barrier: the same value for every thread
  }
  if (ok) {
    write_A1(1);
    tc::fence_proxy_async();
    __syncthreads();
    if (warp == 0) {
      const uint32_t b1 = bbase + 2u * S::N1 * S::K1 * 4u;
      mma_3xtf32_2(tbase + 2 * S::N1, aHs, aLs, b1, S::N1, S::K1, idesc1w, idesc1);
      tc::mma_commit_warp(&mbar[1]);
      n_c1 = 2;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 1, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
  }
  if (ok) {
    // B1 is no longer read: fetch B2 into the same buffer, overlapped with the epilogue
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(&mbar[0], (uint32_t)(S::B2 * sizeof(float)));
      tc::bulk_g2s(sB, gbasis + (size_t)m * S::BLOCK + S::B1, (uint32_t)(S::B2 * sizeof(float)), &mbar[0]);
      n_tma = 2;
    }
    // ---- phase 3: D1 -> staging sRes[g][n-m][member, re/im]; zero the A2 operands
    {
      const int quarter = warp & 3, par = warp >> 2;
      const int row = quarter * 32 + lane;
      const int gq = row >> 4, btc = row & 15;
      const int Cp = par ? C1 : C0;
#pragma unroll
      for (int c0 = 0; c0 < S::N1; c0 += 16) {
        float v[16], v1[16];
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * par * S::N1 + c0), v);
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((2 * par + 1) * S::N1 + c0), v1);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += v1[i];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = c0 + i;
          if (c < Cp) sRes[(gq * CNT + (par + 2 * c)) * 16 + btc] = v[i];
        }
      }
    }
    for (int i = threadIdx.x; i < S::RES0; i += blockDim.x) sA[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 4: spectral epilogue -> A2 operands [par][hi, lo][112 rows][K2]
    for (int t = threadIdx.x; t < MT * cnt; t += blockDim.x) {
      const int bti = t % MT, kk = t / MT, n = m + kk;
      const int par = kk & 1, c = kk >> 1;
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
      float* aH = sA + (size_t)(2 * par) * S::A2;
      float* aL = aH + S::A2;
#pragma unroll
      for (int q = 0; q < 7; ++q)
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
    // ---- phase 5: GEMM2, both parities (rows 112..127 read the staging area and are ignored)
    // Warp 0 issues the MMAs first; then every thread issues the global loads
    // of its write-out pairs, whose latency overlaps the GEMM.
    if (warp == 0) {
      const bool good = tc::mbar_wait_bounded_warp(&mbar[0], 1, basis.wait_limit);
      if (!good) *sflag = 1;
      if (good) {
        for (int par = 0; par < 2; ++par) {
          const uint32_t a2 = aHs + (uint32_t)(2 * par * S::A2) * 4u;
          const uint32_t bp = bbase + (uint32_t)(2 * par * S::N2 * S::K2) * 4u;
          mma_3xtf32(tbase + 2 * S::N1 + par * S::N2, a2, a2 + S::A2 * 4, bp, bp + S::N2 * S::K2 * 4, S::K2,
                     idesc2);
        }
      }
      tc::mma_commit_warp(&mbar[2]);
      n_c2 = 1;
    }
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
      for (int cc = 0; cc < JH / 16; ++cc) {
        const int col0 = half * JH + cc * 16;
        float E[16], O[16];
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * S::N1 + col0), E);
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * S::N1 + S::N2 + col0), O);
        if (active) {
          float* o = Out + (size_t)(q * MT + bti) * S::OST + comp;
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
  if (warp == 0) tc::tmem_dealloc(tbase, S::TMEM_COLS);
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
__host__ __device__ constexpr int adj_hslot(int q) {  // H result of GEMM2' row group q, or -1
  return q == 0 ? 0 : q == 2 ? 1 : q == 3 ? 2 : q == 4 ? 3 : -1;
}
}  // namespace

size_t spec_tc_adj_smem_bytes(int M) {
  if (M == 106) return spec_tc106_adj_smem_bytes();
  return tc_dispatch(M, [](auto S) { return (size_t)(S.AA + S.B1 + S.COEF) * sizeof(float) + 256; });
}

template <class S>
__global__ void __launch_bounds__(256, S::MINB) k_spectral_adj_tc(const __grid_constant__ SpecLaunch<float> L,
                                                                  const __grid_constant__ TcBasis basis, int* err) {
  typedef float T;
  typedef float2 T2;
  constexpr int NKADJ = 8;
  constexpr int MT = S::MT, J = S::J, JH = S::JH, CNT = S::CNT;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  pdl_trigger();
  int idx;
  const SpecGroup<T>& G = pick_group(L, idx);
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  const float* gbasis = basis.p[gi];
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

  float* sA = (float*)smem_raw;            // staged lambda | A1' | A2' + D1' staging | output staging
  float* sB = sA + S::AA;                  // B1', then B2'; after GEMM2' the per-pair Phibar terms
  float* sRes = sA + S::ARES0;
  float* sig = sB + S::B1;
  float* sigP = sig + MT * CNT;
  float* sigm1 = sigP + MT * CNT;
  float* sigPm1 = sigm1 + MT * CNT;
  float* tcmn = sigPm1 + MT * CNT;
  uint64_t* mbar = (uint64_t*)(((uintptr_t)(tcmn + MT * CNT) + 15) & ~(uintptr_t)15);  // [4]
  uint32_t* tslot = (uint32_t*)(mbar + 4);
  int* sflag = (int*)(tslot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int n_tma = 0, n_in = 0, n_c1 = 0, n_c2 = 0;

  // ---- phase 0: barriers; bulk copies of B1' and (after the wait for the
  // previous kernel in the stream) of lambda_Y (5 fields); TMEM; coefficients
  if (threadIdx.x == 0) {
    *sflag = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) tc::mbar_init(&mbar[q], 1);
    tc::fence_mbar_init();
    tc::mbar_expect_tx(&mbar[0], (uint32_t)(S::B1 * sizeof(float)));
    tc::bulk_g2s(sB, gbasis + (size_t)m * S::BLOCK, (uint32_t)(S::B1 * sizeof(float)), &mbar[0]);
    n_tma = 1;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, S::TMEM_COLS);
    tc::tmem_relinquish();
  }
  pdl_wait();
  if (threadIdx.x == 0) {
    const uint32_t row_bytes = (uint32_t)(mt * J * sizeof(T2));
    tc::mbar_expect_tx(&mbar[3], row_bytes * S::ANIN);
#pragma unroll
    for (int q = 0; q < S::ANIN; ++q)
      tc::bulk_g2s(sA + (size_t)q * MT * J * 2, G.lamY + (size_t)q * FS + ((size_t)m * G.B + b0) * J, row_bytes,
                   &mbar[3]);
    n_in = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  // ---- phase 1: symmetrised lambda_Y of (member, j'); warp tasks of 4 members x 8 j'
  int jp[S::NPAIR], bt[S::NPAIR];
  bool has[S::NPAIR];
#pragma unroll
  for (int k = 0; k < S::NPAIR; ++k) {
    const int task = warp + 8 * k;
    has[k] = task < S::NTASK;
    const int jb = has[k] ? task % (JH / 8) : 0, mb = has[k] ? task / (JH / 8) : 0;
    jp[k] = jb * 8 + (lane & 7);
    bt[k] = mb * 4 + (lane >> 3);
  }
  T2 ys[S::NPAIR][S::ANIN], ya[S::NPAIR][S::ANIN];
  // write-out: thread -> member wbt, latitudes wj, wj + 1 (16-byte accesses)
  int wbt[S::NWPAIR], wj[S::NWPAIR];
#pragma unroll
  for (int k = 0; k < S::NWPAIR; ++k) {
    const int q = threadIdx.x + 256 * k;
    wbt[k] = q < MT * J / 2 ? q / (J / 2) : MT;
    wj[k] = 2 * (q % (J / 2));
  }
  AdjRowsIn<T> pin[S::NWPAIR];  // its inputs, loaded ahead of GEMM2'
  bool ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[3], 0, basis.wait_limit) : true;
  ok = __syncthreads_and(ok);
  if (ok) {
    const T2* stg = (const T2*)sA;
#pragma unroll
    for (int k = 0; k < S::NPAIR; ++k)
#pragma unroll
      for (int f = 0; f < S::ANIN; ++f) {
        if (has[k] && bt[k] < mt) {
          const T2 u = stg[(f * MT + bt[k]) * J + jp[k]], v = stg[(f * MT + bt[k]) * J + (J - 1 - jp[k])];
          ys[k][f] = cadd(u, v);
          ya[k][f] = csub(u, v);
        } else {
          ys[k][f] = mk<T2>(0, 0);
          ya[k][f] = ys[k][f];
        }
      }
  }
  // parity 0: the P groups take the symmetric sums, the H groups the antisymmetric ones
  auto write_A1 = [&](int par) {
    float* aH = sA;
    float* aL = sA + S::ROWS * S::K1;
#pragma unroll
    for (int k = 0; k < S::NPAIR; ++k) {
      if (!has[k]) continue;
#pragma unroll
      for (int gq = 0; gq < 7; ++gq) {
        const bool hg = gq >= 5;
        const int f = hg ? gq - 2 : gq;  // H groups carry lambda U, V
        const T2 v = hg ? (par ? ys[k][f] : ya[k][f]) : (par ? ya[k][f] : ys[k][f]);
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          const int row = gq * 16 + bt[k] * 2 + comp;
          float hi, lo;
          tc::split_tf32(comp ? v.y : v.x, hi, lo);
          aH[tc::cm_index(row, hg ? JH + jp[k] : jp[k], S::K1)] = hi;
          aL[tc::cm_index(row, hg ? JH + jp[k] : jp[k], S::K1)] = lo;
          aH[tc::cm_index(row, hg ? jp[k] : JH + jp[k], S::K1)] = 0.f;
          aL[tc::cm_index(row, hg ? jp[k] : JH + jp[k], S::K1)] = 0.f;
        }
      }
    }
  };
  const uint32_t idesc1 = tc::idesc_tf32(S::ROWS, S::N1), idesc1w = tc::idesc_tf32(S::ROWS, 2 * S::N1);
  const uint32_t idesc2 = tc::idesc_tf32(S::ROWS, S::N2);
  const uint32_t aHs = tc::smem_u32(sA), aLs = aHs + (uint32_t)(S::ROWS * S::K1 * 4);
  const uint32_t bbase = tc::smem_u32(sB);

  // ---- phase 2: GEMM1', parity 0 then parity 1
  if (ok) {
    __syncthreads();  // the staged lambda is read: A1' overwrites it
    write_A1(0);
    tc::fence_proxy_async();
    __syncthreads();
    if (warp == 0) {  // warp-collective MMA issue
      const bool good = tc::mbar_wait_bounded_warp(&mbar[0], 0, basis.wait_limit);
      if (!good) *sflag = 1;
      if (good) mma_3xtf32_2(tbase, aHs, aLs, bbase, S::N1, S::K1, idesc1w, idesc1);
      tc::mma_commit_warp(&mbar[1]);
      n_c1 = 1;
    }
    // the epilogue's per-(member, n) coefficients, gathered while the MMAs run
    load_spec_coefs<T>(G, cfg.diffflag != 0, m, b0, mt, MT, cnt, CNT, sig, sigP, sigm1, sigPm1, tcmn);
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 0, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ok = ok && !*sflag;
  }
  if (ok) {
    write_A1(1);
    tc::fence_proxy_async();
    __syncthreads();
    if (warp == 0) {
      const uint32_t b1 = bbase + 2u * S::N1 * S::K1 * 4u;
      mma_3xtf32_2(tbase + 2 * S::N1, aHs, aLs, b1, S::N1, S::K1, idesc1w, idesc1);
      tc::mma_commit_warp(&mbar[1]);
      n_c1 = 2;
    }
    ok = threadIdx.x == 0 ? tc::mbar_wait_bounded(&mbar[1], 1, basis.wait_limit) : true;
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
  }
  if (ok) {
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(&mbar[0], (uint32_t)(S::B2 * sizeof(float)));
      tc::bulk_g2s(sB, gbasis + (size_t)m * S::BLOCK + S::B1, (uint32_t)(S::B2 * sizeof(float)), &mbar[0]);
      n_tma = 2;
    }
    // ---- phase 3: D1' -> sRes[q][n-m][member, re/im]; zero the A2' operands
    {
      const int quarter = warp & 3, par = warp >> 2;
      const int row = quarter * 32 + lane;
      const int gq = row >> 4, btc = row & 15;
      const int Cp = par ? C1 : C0;
#pragma unroll
      for (int c0 = 0; c0 < S::N1; c0 += 16) {
        float v[16], v1[16];
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * par * S::N1 + c0), v);
        tc::tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((2 * par + 1) * S::N1 + c0), v1);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += v1[i];
        if (gq < 7) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int c = c0 + i;
            if (c < Cp) sRes[(gq * CNT + (par + 2 * c)) * 16 + btc] = v[i];
          }
        }
      }
    }
    for (int i = threadIdx.x; i < S::ARES0; i += blockDim.x) sA[i] = 0.f;
    tc::fence_before_sync();
    __syncthreads();
    // ---- phase 4: transposed wind inversion, n(n+1), hyperdiffusion -> A2' [par][hi, lo][128][K2]
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
      float* aH = sA + (size_t)(2 * par) * S::AA2;
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
    // ---- phase 5: GEMM2', both parities; write-out inputs loaded meanwhile (after the MMA issue)
    if (warp == 0) {
      const bool good = tc::mbar_wait_bounded_warp(&mbar[0], 1, basis.wait_limit);
      if (!good) *sflag = 1;
      if (good) {
        for (int par = 0; par < 2; ++par) {
          const uint32_t a2 = aHs + (uint32_t)(2 * par * S::AA2) * 4u;
          const uint32_t bp = bbase + (uint32_t)(2 * par * S::N2 * S::K2) * 4u;
          mma_3xtf32(tbase + 2 * S::N1 + par * S::N2, a2, a2 + S::AA2 * 4, bp, bp + S::N2 * S::K2 * 4, S::K2,
                     idesc2);
        }
      }
      tc::mma_commit_warp(&mbar[2]);
      n_c2 = 1;
    }
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k)
      if (wbt[k] < mt) adj_load_rows<T>(G, incr, FS, ((size_t)m * G.B + b0 + wbt[k]) * J + wj[k], pin[k]);
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
      for (int cc = 0; cc < JH / 16; ++cc) {
        const int col0 = half * JH + cc * 16;
        float E[16], O[16];
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * S::N1 + col0), E);
        tc::tmem_ld16(tbase + lanes + (uint32_t)(2 * S::N1 + S::N2 + col0), O);
        if (slot >= 0) {
          float* o = Out + (size_t)(slot * MT + bti) * S::OST + comp;
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
    // ---- phase 7: transposed combination -> lambda of the state fields; the
    // Phibar gradient terms of each latitude pair go to sgp (the B buffer is free)
    float* sgp = sB;  // [MT][J / 2]
#pragma unroll
    for (int k = 0; k < S::NWPAIR; ++k) {
      if (wbt[k] < mt) {
        const int b = b0 + wbt[k];
        const size_t o = ((size_t)m * G.B + b) * J + wj[k];
        auto ld = [&](int q, int e) {
          return *(const float2*)&Out[(size_t)(q * MT + wbt[k]) * S::OST + 2 * (wj[k] + e)];
        };
        const T gp = adj_store_rows<T, NKADJ>(G, cfg, incr, FS, o, m, b, wj[k], ld, pin[k]);
        sgp[wbt[k] * (J / 2) + wj[k] / 2] = gp;
      }
    }
    __syncthreads();
    if (G.grad && warp < mt) {  // one warp per member, reduced in a fixed order
      float acc = 0.f;
      for (int i = lane; i < J / 2; i += 32) acc += sgp[warp * (J / 2) + i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) atomicAdd(&G.grad[G_PHIBAR * G.B + b0 + warp], (double)acc);
    }
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
  if (warp == 0) tc::tmem_dealloc(tbase, S::TMEM_COLS);
}

void spec_tc_set_attributes() {
  cudaFuncSetAttribute(k_spectral_tc<Tc42>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_tc_smem_bytes(42));
  cudaFuncSetAttribute(k_spectral_adj_tc<Tc42>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)spec_tc_adj_smem_bytes(42));
  cudaFuncSetAttribute(k_spectral_tc<Tc63>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_tc_smem_bytes(63));
  cudaFuncSetAttribute(k_spectral_adj_tc<Tc63>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)spec_tc_adj_smem_bytes(63));
  spec_tc106_set_attributes();
}

// One launch per truncation: L holds only the groups of truncation M (the
// others have no members, so no CTAs).
cudaError_t launch_spec_tc(int M, const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                           cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  if (M == 106) return launch_spec_tc106(L, nblocks, basis, err, s);
  cudaError_t e = M == 63 ? launch_pdl(k_spectral_tc<Tc63>, nblocks, 256, spec_tc_smem_bytes(63), s, true, L, basis, err)
                          : launch_pdl(k_spectral_tc<Tc42>, nblocks, 256, spec_tc_smem_bytes(42), s, true, L, basis, err);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_spec_adj_tc(int M, const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                               cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  if (M == 106) return launch_spec_adj_tc106(L, nblocks, basis, err, s);
  cudaError_t e =
      M == 63 ? launch_pdl(k_spectral_adj_tc<Tc63>, nblocks, 256, spec_tc_adj_smem_bytes(63), s, true, L, basis, err)
              : launch_pdl(k_spectral_adj_tc<Tc42>, nblocks, 256, spec_tc_adj_smem_bytes(42), s, true, L, basis, err);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace swp
