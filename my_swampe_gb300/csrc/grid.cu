// K2: the per-latitude grid-space half of a time step, its set-up, output and
// adjoint variants.  One CTA owns one ensemble member and a block of JB
// latitude rows.  For each row it
//   * turns truncated Fourier coefficients (m = 0..M) into I real grid values
//     with a half-length complex FFT (the reference's ifft of a Hermitian-
//     filled array followed by jnp.real, spectral_transform.py:331-348 and
//     model.py:973-977; the m=0 imaginary part is dropped exactly as real() does),
//   * evaluates the grid-space terms: A..E (initial_conditions.py:242-292),
//     Newtonian relaxation Q and drag F, G (forcing.py:14-155, computed whenever
//     the run is forced, model.py:560-603),
//   * and returns them to truncated Fourier space (fft(x/I)[:M+1],
//     spectral_transform.py:309-328) with a half-length complex FFT.
// Mixed-radix Stockham passes (radix 8/4/3/5) run in shared memory on
// transforms padded to L+1 entries (bank-conflict-free across a warp).
// Fourier rows are staged through shared memory.  The Fourier fields keep the
// latitude index fastest, so a CTA's rows of one (field, m) are a contiguous
// JB-element run.  The step, adjoint-step and tangent-step modes copy them
// with 16-byte cp.async issued at the start of the CTA; the kernels are bound
// by memory instructions in flight per SM rather than by bytes.
// The kernel is specialised per mode at compile time.
#include "grid_common.cuh"

namespace swp {

// transforms per row held simultaneously in each mode
__host__ __device__ constexpr int grid_ntr(int mode) {
  return mode == GM_ADJ_STEP ? 12 : (mode == GM_WINDS || mode == GM_FWD2) ? 2 : 8;
}

template <typename T>
size_t grid_smem_bytes(int M, int J, int I, int JB, int mode) {
  (void)M; (void)J;
  int LS = I / 2 + 1;
  size_t ntr = (size_t)grid_ntr(mode) * JB;
  size_t buf = ntr * LS * sizeof(typename cplx<T>::type);
  // two transform buffers, the dayside row, the twiddles (L + (L+1)), reductions
  return 2 * buf + (size_t)I * sizeof(T) + 16 + (size_t)(I + 1) * sizeof(typename cplx<T>::type) + 16 +
         8 * NGRAD * sizeof(double);
}
template size_t grid_smem_bytes<double>(int, int, int, int, int);
template size_t grid_smem_bytes<float>(int, int, int, int, int);

// Per-CTA context shared by the mode bodies.  The grid sizes are compile-time
// (one instantiation per truncation), so every index division in the hot
// loops is by a constant.
template <typename T, int M_, int JB_>
struct GridCtx {
  typedef typename cplx<T>::type T2;
  static constexpr int M = M_, J = trunc_J(M_), I = trunc_I(M_), L = I / 2, LS = L + 1, JB = JB_;
  const GridGroup<T>* G;
  int B, b, j0;
  size_t FS, PS;
  T2* bufA;
  T2* bufB;
  T* sday;
  const T2* twL;   // shared-memory copies of the geometry's twiddles
  const T2* twI;
  double* sred;
  T invI;
};

// Unforced runs (test 1, 2): the forcing terms PhiF, F, G are zero
// (model.py:601-603).  Written explicitly for the CTA's rows, since an
// out-of-place step or a caller's fresh buffer would leave them undefined.
template <typename T, typename C>
__device__ __forceinline__ void zero_forcing_rows(const C& c, typename cplx<T>::type* four) {
  typedef typename cplx<T>::type T2;
  constexpr int n1 = C::M + 1;
  for (int t = threadIdx.x; t < 3 * n1 * C::JB; t += blockDim.x) {
    const int r = t % C::JB, k = (t / C::JB) % n1, q = t / (C::JB * n1);
    four[(F_PHIF + q) * c.FS + ((size_t)k * c.B + c.b) * C::J + c.j0 + r] = mk<T2>(0, 0);
  }
}

// Stage the rows j0..j0+JB-1 of `nf` Fourier fields of member b into `stage`
// ([f][r][m], m fastest; the global reads are JB-long contiguous runs).  The
// field pointers go through a shared-memory table rather than a local array.
// With scale0 / scale (per field, may be null for 1) the staged value of m = 0
// is multiplied by scale0[f] and those of m >= 1 by scale[f] (the C2R bin scales).
template <typename T, typename C>
__device__ __forceinline__ void stage_rows(const C& c, const typename cplx<T>::type* const* src, int nf,
                                           typename cplx<T>::type* stage, const T* scale0 = nullptr,
                                           const T* scale = nullptr) {
  typedef typename cplx<T>::type T2;
  __shared__ const T2* s_src[16];
  __shared__ T s_sc[2][16];
  if (threadIdx.x < 16) {
    const bool on = (int)threadIdx.x < nf;
    s_src[threadIdx.x] = on ? src[threadIdx.x] : nullptr;
    s_sc[0][threadIdx.x] = (on && scale0) ? scale0[threadIdx.x] : (T)1;
    s_sc[1][threadIdx.x] = (on && scale) ? scale[threadIdx.x] : (T)1;
  }
  __syncthreads();
  const bool scaled = scale0 != nullptr;
  constexpr int n1 = C::M + 1;
  // batches of 8 loads in flight before their shared-memory stores (the compiler
  // cannot move a global load above a store through a possibly aliasing pointer)
  constexpr int NB = 8;
  const int total = nf * n1 * C::JB;
  for (int t0 = threadIdx.x; t0 < total; t0 += NB * blockDim.x) {
    T2 v[NB];
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int t = t0 + u * blockDim.x;
      if (t < total) {
        const int r = t % C::JB, k = (t / C::JB) % n1, f = t / (C::JB * n1);
        v[u] = s_src[f][((size_t)k * c.B + c.b) * C::J + c.j0 + r];
      }
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int t = t0 + u * blockDim.x;
      if (t < total) {
        const int r = t % C::JB, k = (t / C::JB) % n1, f = t / (C::JB * n1);
        stage[(f * C::JB + r) * n1 + k] = scaled ? cscale(v[u], s_sc[k == 0 ? 0 : 1][f]) : v[u];
      }
    }
  }
}

// The adjoint step's batch 1: lambda of the first nz nonlinear terms (F_A,
// F_B, ...) scaled 1/I at m = 0 and 1/(2I) above it, then the primal eta, Phi,
// U, V unscaled, staged as [f][m][r] (rows fastest, so that one 16-byte
// cp.async moves Rows16 adjacent rows; c2r_transform<..., true> reads this
// layout).  The copies are issued at the start of the CTA, so that their
// latency covers its set-up; adj_stage_finish completes them and applies the
// scales.  Each thread scales exactly the elements it copied (same index loop),
// so it needs only its own copies complete; a block barrier must follow.
template <typename T, typename C>
__device__ __forceinline__ void adj_stage_issue(const C& c, const GridGroup<T>& G, int nz, int nb1,
                                                typename cplx<T>::type* stage) {
  typedef typename cplx<T>::type T2;
  constexpr int n1 = C::M + 1;
  constexpr int EPC = Rows16<T2>::N, RP = C::JB / EPC;
  const int total = nb1 * n1 * RP;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int rp = t % RP, k = (t / RP) % n1, f = t / (RP * n1);
    const int q = f - nz;
    const T2* p = f < nz ? G.lam + (size_t)(F_A + f) * c.FS
                         : G.primal + (size_t)(q == 0 ? F_ETA : q == 1 ? F_PHI : q == 2 ? F_U : F_V) * c.FS;
    cp_async<16>(stage + (f * n1 + k) * C::JB + rp * EPC, p + ((size_t)k * c.B + c.b) * C::J + c.j0 + rp * EPC);
  }
}
template <typename T, typename C>
__device__ __forceinline__ void adj_stage_finish(const C& c, int nz, typename cplx<T>::type* stage) {
  typedef typename cplx<T>::type T2;
  constexpr int n1 = C::M + 1;
  constexpr int EPC = Rows16<T2>::N, RP = C::JB / EPC;
  cp_async_wait_all();
  for (int t = threadIdx.x; t < nz * n1 * RP; t += blockDim.x) {
    const int rp = t % RP, k = (t / RP) % n1, f = t / (RP * n1);
    const T sc = k == 0 ? c.invI : c.invI * (T)0.5;
#pragma unroll
    for (int e = 0; e < EPC; ++e) {
      T2& v = stage[(f * n1 + k) * C::JB + rp * EPC + e];
      v = cscale(v, sc);
    }
  }
}

// The step's fields at staged positions f0 .. f0+nf-1 of `four` (position f
// holds step_field(f - fofs): eta, Phi, U, V, then delta for history runs,
// unless fixed_field >= 0 names the field), unscaled, in the [f][m][r] layout
// of adj_stage_issue, by 16-byte cp.async.  Completed by cp_async_wait_all and
// a block barrier.
__host__ __device__ constexpr int step_field(int f) {
  return f == 0 ? F_ETA : f == 1 ? F_PHI : f == 2 ? F_U : f == 3 ? F_V : F_DELTA;
}
template <typename T, typename C>
__device__ __forceinline__ void step_stage_issue(const C& c, const typename cplx<T>::type* four, int f0, int nf,
                                                 int fixed_field, typename cplx<T>::type* stage, int fofs = 0) {
  typedef typename cplx<T>::type T2;
  constexpr int n1 = C::M + 1;
  constexpr int EPC = Rows16<T2>::N, RP = C::JB / EPC;
  for (int t = threadIdx.x; t < nf * n1 * RP; t += blockDim.x) {
    const int rp = t % RP, k = (t / RP) % n1, f = f0 + t / (RP * n1);
    const int fld = fixed_field >= 0 ? fixed_field : step_field(f - fofs);
    cp_async<16>(stage + (f * n1 + k) * C::JB + rp * EPC,
                 four + (size_t)fld * c.FS + ((size_t)k * c.B + c.b) * C::J + c.j0 + rp * EPC);
  }
}

// C2R of the `nf` x JB staged rows (layout of stage_rows, [f][r][m], or with
// FMR the [f][m][r] layout of the cp.async staging; scales already
// applied): the half-length spectrum Z (c2r_pre) is formed inside the first,
// twiddle-free radix-8 pass, which writes `other`; the remaining passes run in
// place of the staged rows.  Returns the buffer holding x_{2n} + i x_{2n+1}
// ([t][n], stride LS).
template <typename T, typename C, bool FMR = false>
__device__ __forceinline__ typename cplx<T>::type* c2r_transform(const C& c, typename cplx<T>::type* stage, int nf,
                                                                  typename cplx<T>::type* other) {
  typedef typename cplx<T>::type T2;
  constexpr int L = C::L, LS = C::LS, PER = L / 8, n1 = C::M + 1;
  const int ntr = nf * C::JB;
  const FastDiv divt(ntr);
  for (int task = threadIdx.x; task < ntr * PER; task += blockDim.x) {
    const int j = divt(task), t = task - j * ntr;
    const T2* y = FMR ? stage + (size_t)(t / C::JB) * n1 * C::JB + t % C::JB : stage + (size_t)t * n1;
    T2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = c2r_pre<T2, T>(y, FMR ? C::JB : 1, C::M, L, j + r * PER, c.twI, (T)1, (T)1);
    dftR<8, +1>(v);
    T2* dst = other + (size_t)t * LS + j * 8;
#pragma unroll
    for (int r = 0; r < 8; ++r) dst[r] = v[r];
  }
  __syncthreads();
  return cfft_rest_c<+1, L>(other, stage, ntr, c.twL);
}

// Truncated R2C bins of `nf` transforms in `res` (stride LS) written to global
// Fourier fields dst[f] (r fastest).  Bin scale: k == 0 ? s0 : s.
template <typename T, typename C>
__device__ __forceinline__ void write_r2c(const C& c, const typename cplx<T>::type* res, int nf,
                                          typename cplx<T>::type* const* dst, T s0, T s) {
  typedef typename cplx<T>::type T2;
  __shared__ T2* s_dst[16];
  if (threadIdx.x < 16) s_dst[threadIdx.x] = (int)threadIdx.x < nf ? dst[threadIdx.x] : nullptr;
  __syncthreads();
  constexpr int n1 = C::M + 1;
  constexpr int EPC = Rows16<T2>::N, RP = C::JB / EPC;  // rows per 16-byte store, stores per (field, m)
  // unrolled so that several independent bins are in flight per thread
#pragma unroll 4
  for (int t = threadIdx.x; t < nf * n1 * RP; t += blockDim.x) {
    const int rp = t % RP, k = (t / RP) % n1, q = t / (RP * n1);
    T2 v[EPC];
#pragma unroll
    for (int e = 0; e < EPC; ++e)
      v[e] = r2c_post<T2, T>(res + ((size_t)q * C::JB + rp * EPC + e) * C::LS, C::L, k, c.twI, k == 0 ? s0 : s);
    st_rows16(s_dst[q] + ((size_t)k * c.B + c.b) * C::J + c.j0 + rp * EPC, v);
  }
}

// Warp sums in the compute type into per-warp FP64 slots (no shared-memory
// atomics), then one thread per gradient sums the 8 slots and adds to global.
template <typename T>
__device__ void block_add_grads(const T* gacc, double* sred, double* grad, int B, int b) {
  const int warp = threadIdx.x >> 5;
  for (int q = 0; q < NGRAD; ++q) {
    T v = gacc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sred[warp * NGRAD + q] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x < NGRAD && grad) {
    double acc = 0.0;
    for (int w = 0; w < 8; ++w) acc += sred[w * NGRAD + threadIdx.x];
    atomicAdd(&grad[threadIdx.x * B + b], acc);
  }
}

template <typename T, int MODE, int MM, int JBB>
__device__ __forceinline__ void grid_body(const GridLaunch<T>& Lc, const GridGroup<T>& G, int idx) {
  typedef typename cplx<T>::type T2;
  typedef GridCtx<T, MM, JBB> Ctx;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const StepCfg& cfg = Lc.cfg;
  constexpr int J = Ctx::J, I = Ctx::I, L = Ctx::L, LS = Ctx::LS, JB = Ctx::JB, M = Ctx::M;
  Ctx c;
  c.G = &G;
  c.B = G.B;
  c.b = idx / (J / JB);
  c.j0 = (idx % (J / JB)) * JB;
  c.FS = (size_t)(M + 1) * G.B * J;
  c.PS = (size_t)G.B * J * I;
  constexpr int NTR = grid_ntr(MODE);
  c.bufA = (T2*)smem_raw;
  c.bufB = c.bufA + (size_t)NTR * JB * LS;
  c.sday = (T*)(c.bufB + (size_t)NTR * JB * LS);
  T2* stw = (T2*)(((uintptr_t)(c.sday + I) + 15) & ~(uintptr_t)15);  // twL [L], then twI [L+1]
  c.twL = stw;
  c.twI = stw + L;
  c.sred = (double*)(((uintptr_t)(stw + 2 * L + 1) + 15) & ~(uintptr_t)15);
  c.invI = (T)1 / (T)I;
  // adjoint step: batch 1's rows (the lambda of nz nonlinear terms with F, G
  // taken from B, A inside a forced sweep, then 4 primal fields) are copied
  // before the set-up below, which their latency then covers
  const bool adj_tied = MODE == GM_ADJ_STEP && cfg.test == 0 && cfg.lam_fg_tied != 0;
  const int adj_nz = adj_tied ? 6 : (cfg.test == 0 ? 8 : 5);
  if (MODE == GM_ADJ_STEP) adj_stage_issue<T>(c, G, adj_nz, adj_nz + 4, c.bufB);
  // step: likewise eta, Phi, U, V (and delta for the history); the diagnostic
  // Phi row, which depends on the member's blow-up flag, follows the set-up
  const int step_nfix = G.hist ? 5 : 4;
  if (MODE == GM_STEP) step_stage_issue<T>(c, G.four, 0, step_nfix, -1, c.bufB);
  // tangent step: the primal eta, Phi, U, V, then their tangents
  if (MODE == GM_TL_STEP) {
    step_stage_issue<T>(c, G.primal, 0, 4, -1, c.bufB);
    step_stage_issue<T>(c, G.four, 4, 4, -1, c.bufB, 4);
  }
  for (int i = threadIdx.x; i < I; i += blockDim.x) c.sday[i] = G.g.dayc[i];
  for (int i = threadIdx.x; i < 2 * L + 1; i += blockDim.x) stw[i] = i < L ? G.g.twL[i] : G.g.twI[i - L];
  if (threadIdx.x == 0) { c.sred[0] = 0.0; c.sred[1] = 1e300; c.sred[2] = 1e300; c.sred[3] = -1e300; }

  const int B = G.B, b = c.b, j0 = c.j0;
  const size_t FS = c.FS, PS = c.PS;
  const Geom<T>& g = G.g;
  // per-member scalars, formed once per CTA by thread 0 (FP64 parameters in,
  // compute type out) and shared: FP64 arithmetic replicated over all 256
  // threads of every CTA would load GB300's small FP64 pipe
  __shared__ T s_par[7];     // Phibar, 1/taurad, 1/taudrag, DPhieq, w_curr, w_mid, w_winds
  __shared__ int s_flag[2];  // no drag (taudrag == -1), member blown up
  __shared__ T s_dpar[NGRAD];  // tangent-linear modes: d(taurad, taudrag, DPhieq, Phibar)
  __shared__ T s_dw[2];        // tangent step and output: tangents of w_curr, w_mid
  if (threadIdx.x == 0) {
    if (MODE == GM_TL_STEP || MODE == GM_TL_INIT)
      for (int q = 0; q < NGRAD; ++q) s_dpar[q] = (T)G.dpar[q * B + b];
    s_dw[0] = G.dw ? (T)G.dw[b] : (T)0;
    s_dw[1] = G.dw ? (T)G.dw[B + b] : (T)0;
    const double Pb = G.par[P_PHIBAR * B + b], tr = G.par[P_TAURAD * B + b];
    const double td = G.par[P_TAUDRAG * B + b], DPe = G.par[P_DPHIEQ * B + b];
    const double wc = G.member ? G.member[MS_WCURR * B + b] : 0.0;
    const double wm = G.member ? G.member[MS_WMID * B + b] : 0.0;
    s_par[0] = (T)Pb; s_par[1] = (T)(1.0 / tr); s_par[2] = (T)(1.0 / td); s_par[3] = (T)DPe;
    s_par[4] = (T)wc; s_par[5] = (T)wm;
    // the winds of a stepped member are band-limited (the RAW filter leaves
    // them alone while it moves eta, delta, Phi of the new level)
    const bool stepped = G.member && G.member[MS_UPDATED * B + b] != 0.0;
    s_par[6] = stepped ? (T)0 : (T)wc;
    s_flag[0] = td == -1.0;
    s_flag[1] = (cfg.diagnostics && G.member) ? (G.member[MS_DEAD * B + b] != 0.0) : 0;
  }
  __syncthreads();
  Physics<T> ph;
  ph.Pb = s_par[0]; ph.itr = s_par[1]; ph.itd = s_par[2]; ph.DPe = s_par[3];
  ph.nodrag = s_flag[0] != 0; ph.forced = (cfg.test == 0);
  const T invI = c.invI;
  T2* bufA = c.bufA;
  T2* bufB = c.bufB;

  if (MODE == GM_STEP || MODE == GM_OUTPUT || MODE == GM_WINDS) {
    // ------------------------------------------------ Fourier -> physical
    const T wcur = s_par[4], wmid = s_par[5], wuv = s_par[6];
    const bool dead = s_flag[1] != 0;
    int fl[8], nf = 0;
    if (MODE == GM_STEP) {
      fl[nf++] = F_ETA; fl[nf++] = F_PHI; fl[nf++] = F_U; fl[nf++] = F_V;
      if (G.hist) fl[nf++] = F_DELTA;
      if (cfg.diagnostics) fl[nf++] = dead ? F_PHI : F_PHI_MID;
    } else if (MODE == GM_OUTPUT) {
      fl[nf++] = F_ETA; fl[nf++] = F_DELTA; fl[nf++] = F_PHI; fl[nf++] = F_U; fl[nf++] = F_V;
      fl[nf++] = F_ETA_MID; fl[nf++] = F_DELTA_MID; fl[nf++] = F_PHI_MID;
    } else {
      fl[nf++] = F_U; fl[nf++] = F_V;
    }
    const T2* src[8];
    T wv[8], dwv[8];
    int rfv[8];
#pragma unroll
    for (int f = 0; f < 8; ++f) {
      wv[f] = (T)0;
      dwv[f] = (T)0;
      rfv[f] = 0;
      src[f] = nullptr;
      if (f < nf) {
        int fld = fl[f];
        src[f] = G.four + fld * FS;
        int rf = -1;
        if (fld == F_ETA || fld == F_ETA_MID) rf = R_ETA;
        else if (fld == F_DELTA || fld == F_DELTA_MID) rf = R_DELTA;
        else if (fld == F_PHI || fld == F_PHI_MID) rf = R_PHI;
        else if (fld == F_U) rf = R_U;
        else if (fld == F_V) rf = R_V;
        const bool is_mid = fld == F_ETA_MID || fld == F_DELTA_MID || fld == F_PHI_MID;
        T w = is_mid ? wmid : wcur;
        // tangent output: the weights' own tangents times the primal residual
        // (zero for the winds, whose weight is zero once a member has stepped)
        T dwt = (G.resid_p && rf >= 0 && rf <= R_PHI) ? s_dw[is_mid ? 1 : 0] : (T)0;
        if (fld == F_U || fld == F_V) w = cfg.test == 1 ? (T)1 : wuv;  // test 1: fixed initial winds (model.py:979-983)
        if (rf >= 0 && G.resid && (w != (T)0 || dwt != (T)0)) { wv[f] = w; dwv[f] = dwt; rfv[f] = rf; }
      }
    }
    if (MODE == GM_STEP) {
      // the copies issued at the start of the CTA, plus the diagnostic row
      if (cfg.diagnostics) step_stage_issue<T>(c, G.four, step_nfix, 1, dead ? F_PHI : F_PHI_MID, bufB);
      cp_async_wait_all();
    } else {
      __syncthreads();
      stage_rows<T>(c, src, nf, bufB);
    }
    __syncthreads();
    T2* zin = MODE == GM_STEP ? c2r_transform<T, Ctx, true>(c, bufB, nf, bufA) : c2r_transform<T>(c, bufB, nf, bufA);
    T2* zout = (zin == bufA) ? bufB : bufA;
    // initial-condition residual (non-zero only before a member's first step and
    // for the fixed test-1 winds): added in shared memory, off the hot loop
    bool need_resid = false;
#pragma unroll
    for (int f = 0; f < 8; ++f) need_resid |= (wv[f] != (T)0 || dwv[f] != (T)0);
    if (need_resid) {
      for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
        int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
        T w = (T)0, dwt = (T)0;
        int rf = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (q == f) { w = wv[q]; dwt = dwv[q]; rf = rfv[q]; }
        if (w != (T)0 || dwt != (T)0) {
          const size_t ro = rf * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
          const T* rs = G.resid + ro;
          T2 z = zin[(size_t)fr * LS + n];
          z.x += w * rs[0];
          z.y += w * rs[1];
          if (dwt != (T)0) {
            z.x += dwt * G.resid_p[ro];
            z.y += dwt * G.resid_p[ro + 1];
          }
          zin[(size_t)fr * LS + n] = z;
        }
      }
      __syncthreads();
    }
    double lrms = 0.0, lspin = 1e300, lmin = 1e300, lmax = -1e300;
#pragma unroll 2
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      T vals[8][2];
#pragma unroll
      for (int f = 0; f < 8; ++f) {
        if (f < nf) {
          T2 z = zin[((size_t)f * JB + r) * LS + n];
          vals[f][0] = z.x; vals[f][1] = z.y;
        } else {
          vals[f][0] = vals[f][1] = (T)0;
        }
      }
      if (MODE == GM_OUTPUT || MODE == GM_WINDS) {
#pragma unroll
        for (int f = 0; f < 8; ++f) {
          if (f < nf) {
            T* o = G.phys_out + f * PS + ((size_t)b * J + j) * I + 2 * n;
            o[0] = vals[f][0]; o[1] = vals[f][1];
          }
        }
        continue;
      }
      // GM_STEP: physics on the two points (2n, 2n+1)
      T ihalf = g.ihalf[j];
      T s = g.coslat[j];
      T outs[2][8];
#pragma unroll
      for (int e = 0; e < 2; ++e)
        ph.eval(vals[0][e], vals[1][e], vals[2][e], vals[3][e], ihalf, c.sday[2 * n + e] * s, outs[e]);
      const int nout = ph.forced ? 8 : 5;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nout) zout[((size_t)q * JB + r) * LS + n] = mk<T2>(outs[0][q], outs[1][q]);
      if (G.hist) {
        // history layout [5][B][J][I]: eta, delta, Phi, U, V
        T* base = G.hist + ((size_t)b * J + j) * I + 2 * n;
        base[0] = vals[0][0]; base[1] = vals[0][1];
        base[PS] = vals[4][0]; base[PS + 1] = vals[4][1];
        base[2 * PS] = vals[1][0]; base[2 * PS + 1] = vals[1][1];
        base[3 * PS] = vals[2][0]; base[3 * PS + 1] = vals[2][1];
        base[4 * PS] = vals[3][0]; base[4 * PS + 1] = vals[3][1];
      }
      if (cfg.diagnostics) {
        double aw = g.area[j];
        int fp = G.hist ? 5 : 4;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          double U = vals[2][e], V = vals[3][e];
          lrms += aw * (U * U + V * V);
          lspin = fmin(lspin, sqrt(U * U + V * V));
          double p = fp == 5 ? vals[5][e] : vals[4][e];
          lmin = fmin(lmin, p);
          lmax = fmax(lmax, p);
        }
      }
    }
    if (MODE == GM_OUTPUT || MODE == GM_WINDS) return;
    if (cfg.diagnostics) {
      for (int o = 16; o > 0; o >>= 1) {
        lrms += __shfl_down_sync(0xffffffffu, lrms, o);
        lspin = fmin(lspin, __shfl_down_sync(0xffffffffu, lspin, o));
        lmin = fmin(lmin, __shfl_down_sync(0xffffffffu, lmin, o));
        lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
      }
      if ((threadIdx.x & 31) == 0) {
        atomicAdd(&c.sred[0], lrms);
        atomic_min_d(&c.sred[1], lspin);
        atomic_min_d(&c.sred[2], lmin);
        atomic_max_d(&c.sred[3], lmax);
      }
    }
    __syncthreads();
    if (cfg.diagnostics && threadIdx.x == 0) {
      double* dn = G.diag + (size_t)(cfg.step + 1) * NDIAG * B;
      double* dc = G.diag + (size_t)cfg.step * NDIAG * B;
      atomicAdd(&dn[D_RMS2 * B + b], c.sred[0]);
      atomic_min_d(&dn[D_SPIN * B + b], c.sred[1]);
      atomic_min_d(&dc[D_PHIMIN * B + b], c.sred[2]);
      atomic_max_d(&dc[D_PHIMAX * B + b], c.sred[3]);
    }
    const int nout = ph.forced ? 8 : 5;
    T2* res = cfft_batch_c<-1, L>(zout, zin, nout * JB, c.twL);
    T2* dst[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) dst[q] = G.four + (F_A + q) * FS;
    write_r2c<T>(c, res, nout, dst, invI, invI);
    if (!ph.forced) zero_forcing_rows<T>(c, G.four);
    return;
  }

  if (MODE == GM_TL_STEP) {
    // ------------------------------------------------ tangent of GM_STEP
    // The new level is band-limited (no initial-condition residual): the primal
    // eta, Phi, U, V (G.primal) and their tangents (G.four) go to the grid, the
    // linearised nonlinear terms and forcing come back as tangent Fourier terms.
    cp_async_wait_all();  // the copies issued at the start of the CTA
    __syncthreads();
    T2* zin = c2r_transform<T, Ctx, true>(c, bufB, 8, bufA);
    T2* zout = (zin == bufA) ? bufB : bufA;
    // The RAW filter leaves the initial-condition residual in the curr eta and
    // Phi with weight w_curr (the primal step adds it too); its tangent is
    // w_curr times the tangent residual plus the weight's tangent times the
    // primal residual.  The winds of a stepped member carry none.
    {
      const T wc = s_par[4], dwc = s_dw[0];
      if ((wc != (T)0 || dwc != (T)0) && G.resid_p && G.resid) {
        for (int t = threadIdx.x; t < 2 * JB * L; t += blockDim.x) {
          int n = t % L, fr = t / L, r = fr % JB, q = fr / JB;  // q 0: eta, 1: Phi
          const size_t ro = (q == 0 ? R_ETA : R_PHI) * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
          const T* rp = G.resid_p + ro;
          const T* rt = G.resid + ro;
          T2 zp = zin[((size_t)q * JB + r) * LS + n];
          T2 zt = zin[((size_t)(4 + q) * JB + r) * LS + n];
          zp.x += wc * rp[0];
          zp.y += wc * rp[1];
          zt.x += wc * rt[0] + dwc * rp[0];
          zt.y += wc * rt[1] + dwc * rp[1];
          zin[((size_t)q * JB + r) * LS + n] = zp;
          zin[((size_t)(4 + q) * JB + r) * LS + n] = zt;
        }
        __syncthreads();
      }
    }
    PhysicsTL<T> pt;
    pt.Pb = ph.Pb; pt.itr = ph.itr; pt.itd = ph.itd; pt.DPe = ph.DPe; pt.nodrag = ph.nodrag; pt.forced = ph.forced;
    const int nout = ph.forced ? 8 : 5;
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      T ihalf = g.ihalf[j];
      T s = g.coslat[j];
      T v[8][2];
#pragma unroll
      for (int f = 0; f < 8; ++f) {
        T2 z = zin[((size_t)f * JB + r) * LS + n];
        v[f][0] = z.x; v[f][1] = z.y;
      }
      T outs[2][8];
#pragma unroll
      for (int e = 0; e < 2; ++e)
        pt.eval(v[0][e], v[1][e], v[2][e], v[3][e], v[4][e], v[5][e], v[6][e], v[7][e], ihalf,
                c.sday[2 * n + e] * s, s_dpar, outs[e]);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nout) zout[((size_t)q * JB + r) * LS + n] = mk<T2>(outs[0][q], outs[1][q]);
    }
    __syncthreads();
    T2* res = cfft_batch_c<-1, L>(zout, zin, nout * JB, c.twL);
    T2* dst[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) dst[q] = G.four + (F_A + q) * FS;
    write_r2c<T>(c, res, nout, dst, invI, invI);
    return;
  }

  if (MODE == GM_FWD2) {
    // ------------------------------------------------ physical eta, delta -> Fourier
    __syncthreads();
    for (int t = threadIdx.x; t < 2 * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * LS + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch_c<-1, L>(bufA, bufB, 2 * JB, c.twL);
    T2* dst[2] = {G.four + F_ETA * FS, G.four + F_DELTA * FS};
    write_r2c<T>(c, res, 2, dst, invI, invI);
    return;
  }

  if (MODE == GM_INIT || MODE == GM_TL_INIT) {
    // ------------------------------------------------ physical ICs -> state
    // (GM_TL_INIT: the tangent ICs -> tangent state; the Fourier carries and
    // residuals are linear in the ICs, the nonlinear terms are linearised
    // about the primal ICs in phys_p)
    // batch 1: eta, delta, Phi, U, V -> Fourier curr (+prev, RA carry) and residuals
    __syncthreads();
    const int nf = 5;
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * LS + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch_c<-1, L>(bufA, bufB, nf * JB, c.twL);
    T2* other = (res == bufA) ? bufB : bufA;
    const int n1 = M + 1;
    // unpack into global and keep the truncated rows in `other` ([f][m][r])
    for (int t = threadIdx.x; t < nf * n1 * JB; t += blockDim.x) {
      const int r = t % JB, k = (t / JB) % n1, f = t / (JB * n1);
      T2 v = r2c_post<T2, T>(res + ((size_t)f * JB + r) * LS, L, k, c.twI, invI);
      size_t o = ((size_t)k * B + b) * J + j0 + r;
      const int sf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
      G.four[sf[f] * FS + o] = v;
      if (f < 3) {
        G.four[(f == 0 ? F_ETA_PREV : f == 1 ? F_DELTA_PREV : F_PHI_PREV) * FS + o] = v;
        G.four[(f == 0 ? F_ETA_MID : f == 1 ? F_DELTA_MID : F_PHI_MID) * FS + o] = v;
      }
      other[(f * JB + r) * n1 + k] = v;  // staged layout of build_c2r
    }
    __syncthreads();
    // band-limited reconstruction -> residual = x - C2R(trunc FFT(x))
    T2* zr = c2r_transform<T>(c, other, nf, res);
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      size_t po = f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      const T* x = G.phys_in + po;
      T2 z = zr[(size_t)fr * LS + n];
      G.resid[po] = x[0] - z.x;
      G.resid[po + 1] = x[1] - z.y;
    }
    __syncthreads();
    // batch 2: nonlinear terms and forcing from the raw initial grids (model.py:723-732)
    double lrms = 0.0, lspin = 1e300;
    const int nout = ph.forced ? 8 : 5;
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      size_t po = ((size_t)b * J + j) * I + 2 * n;
      T ihalf = g.ihalf[j];
      T s = g.coslat[j];
      T outs[2][8];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        T eta = G.phys_in[0 * PS + po + e], Phi = G.phys_in[2 * PS + po + e];
        T U = G.phys_in[3 * PS + po + e], V = G.phys_in[4 * PS + po + e];
        if (MODE == GM_TL_INIT) {
          PhysicsTL<T> pt;
          pt.Pb = ph.Pb; pt.itr = ph.itr; pt.itd = ph.itd; pt.DPe = ph.DPe; pt.nodrag = ph.nodrag;
          pt.forced = ph.forced;
          const T* xp = G.phys_p;
          pt.eval(xp[0 * PS + po + e], xp[2 * PS + po + e], xp[3 * PS + po + e], xp[4 * PS + po + e], eta, Phi,
                  U, V, ihalf, c.sday[2 * n + e] * s, s_dpar, outs[e]);
          continue;
        }
        ph.eval(eta, Phi, U, V, ihalf, c.sday[2 * n + e] * s, outs[e]);
        if (cfg.diagnostics) {
          double Ud = U, Vd = V;
          lrms += g.area[j] * (Ud * Ud + Vd * Vd);
          lspin = fmin(lspin, sqrt(Ud * Ud + Vd * Vd));
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nout) bufA[((size_t)q * JB + r) * LS + n] = mk<T2>(outs[0][q], outs[1][q]);
    }
    if (cfg.diagnostics) {
      for (int o = 16; o > 0; o >>= 1) {
        lrms += __shfl_down_sync(0xffffffffu, lrms, o);
        lspin = fmin(lspin, __shfl_down_sync(0xffffffffu, lspin, o));
      }
      if ((threadIdx.x & 31) == 0) { atomicAdd(&c.sred[0], lrms); atomic_min_d(&c.sred[1], lspin); }
    }
    __syncthreads();
    if (cfg.diagnostics && threadIdx.x == 0) {
      atomicAdd(&G.diag[D_RMS2 * B + b], c.sred[0]);
      atomic_min_d(&G.diag[D_SPIN * B + b], c.sred[1]);
    }
    T2* res2 = cfft_batch_c<-1, L>(bufA, bufB, nout * JB, c.twL);
    T2* dst[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) dst[q] = G.four + (F_A + q) * FS;
    write_r2c<T>(c, res2, nout, dst, invI, invI);
    if (!ph.forced) zero_forcing_rows<T>(c, G.four);
    return;
  }

  if (MODE == GM_ADJ_STEP || MODE == GM_ADJ_INIT) {
    // ---------------------------------------------- adjoint of GM_STEP / GM_INIT
    PhysicsAdj<T> pa;
    pa.Pb = ph.Pb; pa.itr = ph.itr; pa.itd = ph.itd; pa.DPe = ph.DPe; pa.nodrag = ph.nodrag; pa.forced = ph.forced;
    // With forcing on, the Legendre adjoint writes lambda_F = lambda_B and
    // lambda_G = -lambda_A exactly (adj_store_point, forc = 1); inside an
    // adjoint sweep (cfg.lam_fg_tied) F and G are then not transformed but
    // taken from B and A.
    const bool tied = MODE == GM_ADJ_STEP && ph.forced && cfg.lam_fg_tied != 0;
    const int nzl = ph.forced ? 8 : 5;               // lambda fields the physics adjoint reads
    const int nz = tied ? 6 : nzl;                   // of them, transformed here
    const int npr = (MODE == GM_ADJ_STEP) ? 4 : 0;  // primal fields transformed here (eta, Phi, U, V)
    // batch 1: lambda of the nonlinear Fourier terms -> grid (adjoint of fft(x/I)[:M+1]:
    // lambda x_i = (1/I) Re sum_{m=0..M} lambda_m e^{i theta}) and the primal grid fields
    const T2* src[12];
    T s0[12], s1[12];
    const int pf[4] = {F_ETA, F_PHI, F_U, F_V};
    const int nb1 = nz + npr;
#pragma unroll
    for (int f = 0; f < 12; ++f) {
      if (f < nz) { src[f] = G.lam + (F_A + f) * FS; s0[f] = invI; s1[f] = invI * (T)0.5; }
      else if (f < nb1) { src[f] = G.primal + pf[f - nz] * FS; s0[f] = (T)1; s1[f] = (T)1; }
      else { src[f] = nullptr; s0[f] = s1[f] = (T)0; }
    }
    if (MODE == GM_ADJ_STEP) {
      adj_stage_finish<T>(c, nz, bufB);  // the copies issued at the start of the CTA
    } else {
      __syncthreads();
      stage_rows<T>(c, src, nb1, bufB, s0, s1);
    }
    __syncthreads();
    T2* zin = MODE == GM_ADJ_STEP ? c2r_transform<T, Ctx, true>(c, bufB, nb1, bufA) : c2r_transform<T>(c, bufB, nb1, bufA);
    T2* zout = (zin == bufA) ? bufB : bufA;
    T gacc[NGRAD] = {(T)0, (T)0, (T)0, (T)0};
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      T ihalf = g.ihalf[j];
      T s = g.coslat[j];
      T lx[2][4];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        T lz[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          T2 v = q < nz ? zin[((size_t)q * JB + r) * LS + n] : mk<T2>(0, 0);
          lz[q] = e ? v.y : v.x;
        }
        if (tied) { lz[6] = lz[1]; lz[7] = -lz[0]; }
        T eta, Phi, U, V;
        if (MODE == GM_ADJ_STEP) {
          T2 a0 = zin[((size_t)(nz + 0) * JB + r) * LS + n], a1 = zin[((size_t)(nz + 1) * JB + r) * LS + n];
          T2 a2 = zin[((size_t)(nz + 2) * JB + r) * LS + n], a3 = zin[((size_t)(nz + 3) * JB + r) * LS + n];
          eta = e ? a0.y : a0.x; Phi = e ? a1.y : a1.x; U = e ? a2.y : a2.x; V = e ? a3.y : a3.x;
        } else {
          size_t po = ((size_t)b * J + j) * I + 2 * n + e;
          eta = G.phys_in[0 * PS + po]; Phi = G.phys_in[2 * PS + po];
          U = G.phys_in[3 * PS + po]; V = G.phys_in[4 * PS + po];
        }
        pa.eval(eta, Phi, U, V, ihalf, c.sday[2 * n + e] * s, lz, lx[e], gacc);
      }
      if (MODE == GM_ADJ_STEP) {
#pragma unroll
        for (int q = 0; q < 4; ++q) zout[((size_t)q * JB + r) * LS + n] = mk<T2>(lx[0][q], lx[1][q]);
      } else {
        // adjoint of the initial grid fields from the nonlinear terms (eta, delta, Phi, U, V)
        size_t po = ((size_t)b * J + j) * I + 2 * n;
        T* o = G.phys_out;
        o[0 * PS + po] = lx[0][0]; o[0 * PS + po + 1] = lx[1][0];
        o[1 * PS + po] = (T)0;     o[1 * PS + po + 1] = (T)0;
        o[2 * PS + po] = lx[0][1]; o[2 * PS + po + 1] = lx[1][1];
        o[3 * PS + po] = lx[0][2]; o[3 * PS + po + 1] = lx[1][2];
        o[4 * PS + po] = lx[0][3]; o[4 * PS + po + 1] = lx[1][3];
      }
    }
    block_add_grads<T>(gacc, c.sred, G.grad, B, b);
    if (MODE == GM_ADJ_STEP) {
      // adjoint of x = Re(Y_0) + 2 Re sum_{m>=1} Y_m e^{i theta}:  lambda Y_m = c_m sum_i lambda x_i e^{-i theta}
      const int n1 = M + 1;
      // lambda_y field q: eta, delta, Phi, U, V; of them, all but delta (q = 1)
      // add the R2C of transform q - (q > 1) of this batch
      constexpr int EPC = Rows16<T2>::N, RP = JB / EPC;
      constexpr int NY = 5 * (M + 1) * RP;
      constexpr int NU = (NY + 255) / 256;
      // a thread's lambda loads (16 bytes: EPC adjacent rows) are issued before
      // the transforms, so that their latency overlaps them, and before its first store
      T2 lv[NU][EPC];
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int t = threadIdx.x + u * 256;
        if (t < NY) {
          const int rp = t % RP, k = (t / RP) % n1, q = t / (RP * n1);
          const int fy = q == 0 ? F_ETA : q == 1 ? F_DELTA : q == 2 ? F_PHI : q == 3 ? F_U : F_V;
          if (q >= 3 && cfg.adj_zeroed) {  // lambda of U, V: zero after the sweep's first step
#pragma unroll
            for (int e = 0; e < EPC; ++e) lv[u][e] = mk<T2>(0, 0);
          } else {
            ld_rows16(G.lam + (size_t)fy * FS + ((size_t)k * B + b) * J + j0 + rp * EPC, lv[u]);
          }
        }
      }
      T2* res = cfft_batch_c<-1, L>(zout, zin, 4 * JB, c.twL);
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int t = threadIdx.x + u * 256;
        if (t < NY) {
          const int rp = t % RP, k = (t / RP) % n1, q = t / (RP * n1);
          if (q != 1) {
            const int tq = q == 0 ? 0 : q - 1;
#pragma unroll
            for (int e = 0; e < EPC; ++e)
              lv[u][e] = cadd(lv[u][e], r2c_post<T2, T>(res + ((size_t)tq * JB + rp * EPC + e) * LS, L, k, c.twI,
                                                          k == 0 ? (T)1 : (T)2));
          }
          st_rows16(G.lamy + (size_t)q * FS + ((size_t)k * B + b) * J + j0 + rp * EPC, lv[u]);
        }
      }
      return;
    }
    // GM_ADJ_INIT batch 2: adjoint of the Fourier curr carries (fft(x/I)[:M+1]) of the ICs
    __syncthreads();
    const int cf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
    const T2* src2[5];
    T s20[5], s21[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) { src2[f] = G.lam + cf[f] * FS; s20[f] = invI; s21[f] = invI * (T)0.5; }
    stage_rows<T>(c, src2, 5, bufB, s20, s21);
    __syncthreads();
    // the initial state also sets the Fourier prev and mid carries of eta,
    // delta, Phi to curr (GM_INIT): their adjoints add to curr's (nonzero for
    // the explicit scheme, whose steps read the prev level)
    {
      constexpr int n1 = M + 1;
      for (int t = threadIdx.x; t < 3 * n1 * JB; t += blockDim.x) {
        const int r = t % JB, k = (t / JB) % n1, f = t / (JB * n1);
        const size_t o = ((size_t)k * B + b) * J + j0 + r;
        const int pf = f == 0 ? F_ETA_PREV : f == 1 ? F_DELTA_PREV : F_PHI_PREV;
        const int mf = f == 0 ? F_ETA_MID : f == 1 ? F_DELTA_MID : F_PHI_MID;
        const T2 add = cadd(G.lam[pf * FS + o], G.lam[mf * FS + o]);
        T2& dst = bufB[(f * JB + r) * n1 + k];
        dst = cadd(dst, cscale(add, k == 0 ? s20[f] : s21[f]));
      }
    }
    __syncthreads();
    T2* z2 = c2r_transform<T>(c, bufB, 5, bufA);
    for (int t = threadIdx.x; t < 5 * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      size_t po = f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      T2 v = z2[(size_t)fr * LS + n];
      G.phys_out[po] += v.x;
      G.phys_out[po + 1] += v.y;
    }
    return;
  }

  if (MODE == GM_ADJ_OUTPUT) {
    // ---------------------------------------------- seed: lambda of physical curr fields -> Fourier
    __syncthreads();
    const int nf = 5;
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * LS + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch_c<-1, L>(bufA, bufB, nf * JB, c.twL);
    T2* dst[5] = {G.lam + F_ETA * FS, G.lam + F_DELTA * FS, G.lam + F_PHI * FS, G.lam + F_U * FS, G.lam + F_V * FS};
    write_r2c<T>(c, res, nf, dst, (T)1, (T)2);
    return;
  }
}

// JB (latitude rows per CTA) of a truncation and mode: 8 where the mode's two
// transform buffers stay within 72 KB (three or more CTAs per SM), else 4, or
// 2 where even 4 rows would exceed 200 KB (the FP64 adjoint at M=106).
template <typename T>
__host__ __device__ constexpr size_t grid_buf_bytes(int M, int mode, int jb) {
  return (size_t)2 * grid_ntr(mode) * jb * (trunc_I(M) / 2 + 1) * 2 * sizeof(T);
}
template <typename T>
__host__ __device__ constexpr int grid_jb(int M, int mode) {
  return grid_buf_bytes<T>(M, mode, 8) <= 72 * 1024 ? 8 : grid_buf_bytes<T>(M, mode, 4) <= 200 * 1024 ? 4 : 2;
}

// Resident CTAs per SM the register budget is sized for: FP32 adjoint 4 (its
// 52 KB of shared memory allow 4), FP32 forward modes 3 (8 rows per CTA at
// M=42 take 68 KB), FP64 2.
template <typename T, int MODE>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? (MODE == GM_ADJ_STEP ? 4 : 3) : 2)
    k_grid(const __grid_constant__ GridLaunch<T> Lc) {
  pdl_enter();
  int idx;
  const GridGroup<T>& G = pick_ggroup(Lc, idx);
  switch (G.g.M) {  // groups of different truncations share one launch
    case 42: grid_body<T, MODE, 42, grid_jb<T>(42, MODE)>(Lc, G, idx); break;
    case 63: grid_body<T, MODE, 63, grid_jb<T>(63, MODE)>(Lc, G, idx); break;
    default: grid_body<T, MODE, 106, grid_jb<T>(106, MODE)>(Lc, G, idx); break;
  }
}

int grid_rows_per_cta(int M, bool fp64, int mode) { return fp64 ? grid_jb<double>(M, mode) : grid_jb<float>(M, mode); }

// Largest dynamic shared memory the kernel may request: 227 KB per block minus
// the kernel's static shared memory (the pointer tables of stage_rows / write_r2c).
template <typename T, int MODE>
static void set_attr_one() {
  cudaFuncAttributes fa;
  size_t stat = cudaFuncGetAttributes(&fa, k_grid<T, MODE>) == cudaSuccess ? fa.sharedSizeBytes : 1024;
  cudaFuncSetAttribute(k_grid<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(227 * 1024 - stat));
}

void grid_set_attributes() {
  set_attr_one<double, GM_STEP>(); set_attr_one<float, GM_STEP>();
  set_attr_one<double, GM_INIT>(); set_attr_one<float, GM_INIT>();
  set_attr_one<double, GM_OUTPUT>(); set_attr_one<float, GM_OUTPUT>();
  set_attr_one<double, GM_WINDS>(); set_attr_one<float, GM_WINDS>();
  set_attr_one<double, GM_ADJ_STEP>(); set_attr_one<float, GM_ADJ_STEP>();
  set_attr_one<double, GM_ADJ_INIT>(); set_attr_one<float, GM_ADJ_INIT>();
  set_attr_one<double, GM_ADJ_OUTPUT>(); set_attr_one<float, GM_ADJ_OUTPUT>();
  set_attr_one<double, GM_FWD2>(); set_attr_one<float, GM_FWD2>();
  set_attr_one<double, GM_TL_STEP>(); set_attr_one<float, GM_TL_STEP>();
  set_attr_one<double, GM_TL_INIT>(); set_attr_one<float, GM_TL_INIT>();
}

template <typename T>
cudaError_t launch_grid(const GridLaunch<T>& L0, int nblocks0, size_t smem, cudaStream_t s) {
  // rows per CTA and the block decomposition follow the mode (grid_jb)
  (void)nblocks0;
  GridLaunch<T> L = L0;
  int nblocks = 0;
  for (int g = 0; g < L.ng; ++g) {
    GridGroup<T>& G = L.grp[g];
    G.JB = grid_jb<T>(G.g.M, L.mode);
    G.njb = G.g.J / G.JB;
    L.prefix[g] = nblocks;
    nblocks += G.B * G.njb;
  }
  L.prefix[L.ng] = nblocks;
  cudaError_t e = cudaSuccess;
  constexpr bool f32 = std::is_same<T, float>::value;
  switch (L.mode) {
    case GM_STEP: e = launch_pdl(k_grid<T, GM_STEP>, nblocks, 256, smem, s, f32, L); break;
    case GM_INIT: e = launch_pdl(k_grid<T, GM_INIT>, nblocks, 256, smem, s, f32, L); break;
    case GM_OUTPUT: e = launch_pdl(k_grid<T, GM_OUTPUT>, nblocks, 256, smem, s, f32, L); break;
    case GM_WINDS: e = launch_pdl(k_grid<T, GM_WINDS>, nblocks, 256, smem, s, f32, L); break;
    case GM_ADJ_STEP: e = launch_pdl(k_grid<T, GM_ADJ_STEP>, nblocks, 256, smem, s, f32, L); break;
    case GM_ADJ_INIT: e = launch_pdl(k_grid<T, GM_ADJ_INIT>, nblocks, 256, smem, s, f32, L); break;
    case GM_ADJ_OUTPUT: e = launch_pdl(k_grid<T, GM_ADJ_OUTPUT>, nblocks, 256, smem, s, f32, L); break;
    case GM_FWD2: e = launch_pdl(k_grid<T, GM_FWD2>, nblocks, 256, smem, s, f32, L); break;
    case GM_TL_STEP: e = launch_pdl(k_grid<T, GM_TL_STEP>, nblocks, 256, smem, s, f32, L); break;
    case GM_TL_INIT: e = launch_pdl(k_grid<T, GM_TL_INIT>, nblocks, 256, smem, s, f32, L); break;
    default: return cudaErrorInvalidValue;
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}
template cudaError_t launch_grid<double>(const GridLaunch<double>&, int, size_t, cudaStream_t);
template cudaError_t launch_grid<float>(const GridLaunch<float>&, int, size_t, cudaStream_t);

}  // namespace swp
