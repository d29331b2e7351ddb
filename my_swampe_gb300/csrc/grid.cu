// K2: the per-latitude grid-space half of a time step, and its set-up and
// output variants.  One CTA owns one ensemble member and a block of JB
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
// Mixed-radix Stockham passes (radix 8/4/3/5) run in shared memory.
#include "swp_internal.h"
#include <float.h>

namespace swp {

template <typename T> __device__ __forceinline__ T tiny_val();
template <> __device__ __forceinline__ double tiny_val<double>() { return DBL_MIN; }
template <> __device__ __forceinline__ float tiny_val<float>() { return FLT_MIN; }

// number of simultaneously held transforms per row for each mode
__host__ __device__ inline int grid_ntr(int mode) {
  switch (mode) {
    case GM_STEP: return 8;
    case GM_INIT: return 8;
    case GM_OUTPUT: return 8;
    case GM_WINDS: return 2;
    case GM_ADJ_STEP: return 12;
    default: return 8;
  }
}

template <typename T>
size_t grid_smem_bytes(int M, int J, int I, int JB, int mode) {
  int L = I / 2;
  size_t ntr = (size_t)grid_ntr(mode) * JB;
  size_t buf = ntr * L * sizeof(typename cplx<T>::type);
  return 2 * buf + (size_t)I * sizeof(T) + 64 * sizeof(double);
}
template size_t grid_smem_bytes<double>(int, int, int, int, int);
template size_t grid_smem_bytes<float>(int, int, int, int, int);

template <typename T>
__device__ __forceinline__ const GridGroup<T>& pick_ggroup(const GridLaunch<T>& L, int& idx) {
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  idx = blockIdx.x - L.prefix[gi];
  return L.grp[gi];
}

// Build the half-length spectrum Z (length L) of a C2R transform from the
// truncated Fourier row y[0..M] (stride ys).  scale0/scale multiply Y_0 / Y_m.
template <typename T2, typename T>
__device__ __forceinline__ T2 c2r_pre(const T2* y, int ys, int M, int L, int k, const T2* twI, T scale0, T scale) {
  T2 hk = mk<T2>(0, 0), hl = mk<T2>(0, 0);
  if (k == 0) { hk = mk<T2>(y[0].x * scale0, 0); }
  else if (k <= M) { hk = cscale(y[k * ys], scale); }
  int kl = L - k;  // partner index (k=0 -> L, which is > M)
  if (kl >= 1 && kl <= M) hl = cscale(y[kl * ys], scale);
  T2 fe = cadd(hk, cconj(hl));
  T2 fo = cmulc(csub(hk, cconj(hl)), twI[k]);  // * exp(+2 pi i k / I)
  T2 z; z.x = fe.x - fo.y; z.y = fe.y + fo.x;  // fe + i fo
  return z;
}

// Unpack bin k (0..M) of a R2C transform from the half-length spectrum Z.
template <typename T2, typename T>
__device__ __forceinline__ T2 r2c_post(const T2* Z, int L, int k, const T2* twI, T scale) {
  T2 zk = Z[k], zl = cconj(Z[(L - k) % L]);
  T2 e = cscale(cadd(zk, zl), (T)0.5);
  T2 d = csub(zk, zl);
  T2 o; o.x = (T)0.5 * d.y; o.y = (T)-0.5 * d.x;  // d / (2i)
  return cscale(cadd(e, cmul(o, twI[k])), scale);
}

__device__ __forceinline__ void atomic_min_d(double* addr, double v) {
  unsigned long long* a = (unsigned long long*)addr;
  unsigned long long old = *a, assumed;
  int guard = 0;
  while (__longlong_as_double(old) > v && guard++ < 4096) {
    assumed = old;
    old = atomicCAS(a, assumed, __double_as_longlong(v));
    if (old == assumed) break;
  }
}
__device__ __forceinline__ void atomic_max_d(double* addr, double v) {
  unsigned long long* a = (unsigned long long*)addr;
  unsigned long long old = *a, assumed;
  int guard = 0;
  while (__longlong_as_double(old) < v && guard++ < 4096) {
    assumed = old;
    old = atomicCAS(a, assumed, __double_as_longlong(v));
    if (old == assumed) break;
  }
}

template <typename T>
struct Physics {
  T Pb, itr, itd, DPe;
  bool nodrag, forced;
  __device__ void eval(T eta, T Phi, T U, T V, T ihalf, T day_s, T* out) const {
    // ABCDE_init (initial_conditions.py:499-503)
    out[0] = U * eta; out[1] = V * eta; out[2] = U * Phi; out[3] = V * Phi;
    out[4] = (U * U + V * V) * ihalf;
    if (forced) {
      T Phieq = Pb + DPe * day_s;                        // forcing.py:55-60
      T Q = itr * (Phieq - (Phi + Pb));                  // forcing.py:94
      T Qc = Q < (T)0 ? (T)0 : Q;                        // forcing.py:133
      T pt = Phi + Pb;
      T pts = fabs(pt) > (T)0 ? pt : tiny_val<T>();     // forcing.py:139-140
      T r = Qc / pts;
      T Ru = -U * r, Rv = -V * r;
      out[5] = Q;
      out[6] = nodrag ? Ru : Ru - U * itd;               // forcing.py:143-153
      out[7] = nodrag ? Rv : Rv - V * itd;
    }
  }
};

// Adjoint of Physics::eval.  lz = adjoints of (A, B, C, D, E, PhiF, F, G),
// lx = adjoints of (eta, Phi, U, V); gacc accumulates d/d(taurad, taudrag,
// DPhieq, Phibar).  The Q<0 clamp passes no gradient where Q<0 (the
// reference's jnp.where semantics); Phieq's Phibar cancels in Q.
template <typename T>
struct PhysicsAdj {
  T Pb, itr, itd, DPe;
  bool nodrag, forced;
  __device__ void eval(T eta, T Phi, T U, T V, T ihalf, T day_s, const T* lz, T* lx, double* gacc) const {
    T lU = lz[0] * eta + lz[2] * Phi + lz[4] * (T)2 * U * ihalf;
    T lV = lz[1] * eta + lz[3] * Phi + lz[4] * (T)2 * V * ihalf;
    T leta = lz[0] * U + lz[1] * V;
    T lPhi = lz[2] * U + lz[3] * V;
    if (forced) {
      T Phieq = Pb + DPe * day_s;
      T Q = itr * (Phieq - (Phi + Pb));
      bool pos = !(Q < (T)0);
      T Qc = pos ? Q : (T)0;
      T pt = Phi + Pb;
      T pts = fabs(pt) > (T)0 ? pt : tiny_val<T>();
      T r = Qc / pts;
      T lF = lz[6], lG = lz[7];
      T lr = -U * lF - V * lG;
      T itdd = nodrag ? (T)0 : itd;
      lU += lF * (-r - itdd);
      lV += lG * (-r - itdd);
      T lQc = lr / pts;
      T lpts = -lr * r / pts;
      T lQ = lz[5] + (pos ? lQc : (T)0);
      lPhi += -itr * lQ + lpts;
      gacc[G_TAURAD] += (double)lQ * (double)(-Q * itr);
      if (!nodrag) gacc[G_TAUDRAG] += ((double)lF * U + (double)lG * V) * (double)itd * (double)itd;
      gacc[G_DPHIEQ] += (double)lQ * (double)itr * (double)day_s;
      gacc[G_PHIBAR] += (double)lpts;
    }
    lx[0] = leta; lx[1] = lPhi; lx[2] = lU; lx[3] = lV;
  }
};

template <typename T>
__device__ void block_add_grads(double* gacc, double* sred, double* grad, int B, int b) {
  // sred[0..3] must be zero-initialised before the first __syncthreads of the kernel
  for (int q = 0; q < NGRAD; ++q) {
    double v = gacc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sred[q], v);
  }
  __syncthreads();
  if (threadIdx.x < NGRAD && grad) atomicAdd(&grad[threadIdx.x * B + b], sred[threadIdx.x]);
}

template <typename T>
__global__ void __launch_bounds__(256) k_grid(const __grid_constant__ GridLaunch<T> Lc) {
  typedef typename cplx<T>::type T2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int idx;
  const GridGroup<T>& G = pick_ggroup(Lc, idx);
  const StepCfg& cfg = Lc.cfg;
  const int mode = Lc.mode;
  const Geom<T>& g = G.g;
  const int M = g.M, J = g.J, I = g.I, L = g.L, JB = G.JB;
  const int b = idx / G.njb;
  const int j0 = (idx % G.njb) * JB;
  const size_t FS = (size_t)(M + 1) * G.B * J;
  const size_t PS = (size_t)G.B * J * I;  // physical field stride
  const int ntrmax = grid_ntr(mode) * JB;
  T2* bufA = (T2*)smem_raw;
  T2* bufB = bufA + (size_t)ntrmax * L;
  T* sday = (T*)(bufB + (size_t)ntrmax * L);
  // block reductions [0]=rms2 [1]=spin [2]=phimin [3]=phimax (doubles: 16-byte aligned address)
  double* sred = (double*)(((uintptr_t)(sday + I) + 15) & ~(uintptr_t)15);
  for (int i = threadIdx.x; i < I; i += blockDim.x) sday[i] = g.dayc[i];
  if (threadIdx.x == 0) { sred[0] = 0.0; sred[1] = 1e300; sred[2] = 1e300; sred[3] = -1e300; }

  const int B = G.B;
  double Pb = G.par[P_PHIBAR * B + b], tr = G.par[P_TAURAD * B + b];
  double td = G.par[P_TAUDRAG * B + b], DPe = G.par[P_DPHIEQ * B + b];
  Physics<T> ph;
  ph.Pb = (T)Pb; ph.itr = (T)(1.0 / tr); ph.itd = (T)(1.0 / td); ph.DPe = (T)DPe;
  ph.nodrag = (td == -1.0); ph.forced = (cfg.test == 0);
  const T invI = (T)(1.0 / I);
  const double wcur = G.member ? G.member[MS_WCURR * B + b] : 0.0;
  const double wmid = G.member ? G.member[MS_WMID * B + b] : 0.0;
  const bool dead = (cfg.diagnostics && G.member) ? (G.member[MS_DEAD * B + b] != 0.0) : false;

  if (mode == GM_STEP || mode == GM_OUTPUT || mode == GM_WINDS) {
    // ------------------------------------------------ Fourier -> physical
    int fl[8], nf = 0;
    if (mode == GM_STEP) {
      fl[nf++] = F_ETA; fl[nf++] = F_PHI; fl[nf++] = F_U; fl[nf++] = F_V;
      if (G.hist) fl[nf++] = F_DELTA;
      if (cfg.diagnostics) fl[nf++] = dead ? F_PHI : F_PHI_MID;
    } else if (mode == GM_OUTPUT) {
      fl[nf++] = F_ETA; fl[nf++] = F_DELTA; fl[nf++] = F_PHI; fl[nf++] = F_U; fl[nf++] = F_V;
      fl[nf++] = F_ETA_MID; fl[nf++] = F_DELTA_MID; fl[nf++] = F_PHI_MID;
    } else {
      fl[nf++] = F_U; fl[nf++] = F_V;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int k = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T2* y = G.four + fl[f] * FS + (size_t)b * J + (j0 + r);
      bufA[(size_t)fr * L + k] = c2r_pre<T2, T>(y, B * J, M, L, k, g.twI, (T)1, (T)1);
    }
    __syncthreads();
    T2* zin = cfft_batch<+1>(bufA, bufB, L, nf * JB, g.twL);
    T2* zout = (zin == bufA) ? bufB : bufA;
    // residual weights of the initial condition per loaded field
    auto wres = [&](int f, int& rf) -> double {
      rf = -1;
      int fld = fl[f];
      if (fld == F_ETA) rf = R_ETA; else if (fld == F_DELTA) rf = R_DELTA; else if (fld == F_PHI) rf = R_PHI;
      else if (fld == F_U) rf = R_U; else if (fld == F_V) rf = R_V;
      else if (fld == F_ETA_MID) rf = R_ETA; else if (fld == F_DELTA_MID) rf = R_DELTA; else if (fld == F_PHI_MID) rf = R_PHI;
      if (rf < 0) return 0.0;
      if ((fld == F_U || fld == F_V) && cfg.test == 1) return 1.0;  // fixed initial winds (model.py:979-983)
      if (fld == F_ETA_MID || fld == F_DELTA_MID || fld == F_PHI_MID) return wmid;
      return wcur;
    };
    double wv[8]; int rfv[8];
    for (int f = 0; f < nf; ++f) wv[f] = wres(f, rfv[f]);
    double lrms = 0.0, lspin = 1e300, lmin = 1e300, lmax = -1e300;
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      T vals[8][2];
      for (int f = 0; f < nf; ++f) {
        T2 z = zin[((size_t)f * JB + r) * L + n];
        vals[f][0] = z.x; vals[f][1] = z.y;
        if (wv[f] != 0.0 && G.resid) {
          const T* rs = G.resid + rfv[f] * PS + ((size_t)b * J + j) * I + 2 * n;
          vals[f][0] += (T)wv[f] * rs[0];
          vals[f][1] += (T)wv[f] * rs[1];
        }
      }
      if (mode == GM_OUTPUT || mode == GM_WINDS) {
        for (int f = 0; f < nf; ++f) {
          T* o = G.phys_out + f * PS + ((size_t)b * J + j) * I + 2 * n;
          o[0] = vals[f][0]; o[1] = vals[f][1];
        }
        continue;
      }
      // GM_STEP: physics on the two points (2n, 2n+1)
      T ihalf = (T)(1.0 / (2.0 * g.onemu2[j]));
      T s = (T)sqrt(g.onemu2[j]);
      T outs[2][8];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        ph.eval(vals[0][e], vals[1][e], vals[2][e], vals[3][e], ihalf, sday[2 * n + e] * s, outs[e]);
      }
      int nout = ph.forced ? 8 : 5;
      for (int q = 0; q < nout; ++q) zout[((size_t)q * JB + r) * L + n] = mk<T2>(outs[0][q], outs[1][q]);
      if (G.hist) {
        // history layout [5][B][J][I]: eta, delta, Phi, U, V
        const int hf[5] = {0, 4, 1, 2, 3};  // index into vals
        for (int q = 0; q < 5; ++q) {
          T* o = G.hist + q * PS + ((size_t)b * J + j) * I + 2 * n;
          o[0] = vals[hf[q]][0]; o[1] = vals[hf[q]][1];
        }
      }
      if (cfg.diagnostics) {
        int fp = G.hist ? 5 : 4;
        double aw = g.area[j];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          double U = vals[2][e], V = vals[3][e];
          lrms += aw * (U * U + V * V);
          lspin = fmin(lspin, sqrt(U * U + V * V));
          double p = vals[fp][e];
          lmin = fmin(lmin, p);
          lmax = fmax(lmax, p);
        }
      }
    }
    if (mode == GM_OUTPUT || mode == GM_WINDS) return;
    if (cfg.diagnostics) {
      // warp reduce then one atomic per warp into smem, one per block to global
      for (int o = 16; o > 0; o >>= 1) {
        lrms += __shfl_down_sync(0xffffffffu, lrms, o);
        lspin = fmin(lspin, __shfl_down_sync(0xffffffffu, lspin, o));
        lmin = fmin(lmin, __shfl_down_sync(0xffffffffu, lmin, o));
        lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
      }
      if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sred[0], lrms);
        atomic_min_d(&sred[1], lspin);
        atomic_min_d(&sred[2], lmin);
        atomic_max_d(&sred[3], lmax);
      }
    }
    __syncthreads();
    if (cfg.diagnostics && threadIdx.x == 0) {
      double* dn = G.diag + (size_t)(cfg.step + 1) * NDIAG * B;
      double* dc = G.diag + (size_t)cfg.step * NDIAG * B;
      atomicAdd(&dn[D_RMS2 * B + b], sred[0]);
      atomic_min_d(&dn[D_SPIN * B + b], sred[1]);
      atomic_min_d(&dc[D_PHIMIN * B + b], sred[2]);
      atomic_max_d(&dc[D_PHIMAX * B + b], sred[3]);
    }
    int nout = ph.forced ? 8 : 5;
    T2* res = cfft_batch<-1>(zout, zin, L, nout * JB, g.twL);
    for (int t = threadIdx.x; t < nout * JB * (M + 1); t += blockDim.x) {
      int r = t % JB, k = (t / JB) % (M + 1), q = t / (JB * (M + 1));
      T2 v = r2c_post<T2, T>(res + ((size_t)q * JB + r) * L, L, k, g.twI, invI);
      G.four[(F_A + q) * FS + ((size_t)k * B + b) * J + j0 + r] = v;
    }
    return;
  }

  if (mode == GM_ADJ_STEP || mode == GM_ADJ_INIT) {
    // ---------------------------------------------- adjoint of GM_STEP / GM_INIT
    PhysicsAdj<T> pa;
    pa.Pb = ph.Pb; pa.itr = ph.itr; pa.itd = ph.itd; pa.DPe = ph.DPe; pa.nodrag = ph.nodrag; pa.forced = ph.forced;
    const int nz = ph.forced ? 8 : 5;
    const int npr = (mode == GM_ADJ_STEP) ? 4 : 0;  // primal fields transformed here (eta, Phi, U, V)
    if (threadIdx.x < 4) sred[threadIdx.x] = 0.0;
    __syncthreads();
    // batch 1: lambda of the nonlinear Fourier terms -> grid (adjoint of fft(x/I)[:M+1]) and primal grid fields
    const int pf[4] = {F_ETA, F_PHI, F_U, F_V};
    const int nb1 = nz + npr;
    for (int t = threadIdx.x; t < nb1 * JB * L; t += blockDim.x) {
      int k = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      T2 z;
      if (f < nz) {
        const T2* y = G.lam + (F_A + f) * FS + (size_t)b * J + (j0 + r);
        z = c2r_pre<T2, T>(y, B * J, M, L, k, g.twI, invI, invI * (T)0.5);
      } else {
        const T2* y = G.primal + pf[f - nz] * FS + (size_t)b * J + (j0 + r);
        z = c2r_pre<T2, T>(y, B * J, M, L, k, g.twI, (T)1, (T)1);
      }
      bufA[(size_t)fr * L + k] = z;
    }
    __syncthreads();
    T2* zin = cfft_batch<+1>(bufA, bufB, L, nb1 * JB, g.twL);
    T2* zout = (zin == bufA) ? bufB : bufA;
    double gacc[NGRAD] = {0.0, 0.0, 0.0, 0.0};
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      T ihalf = (T)(1.0 / (2.0 * g.onemu2[j]));
      T s = (T)sqrt(g.onemu2[j]);
      T lx[2][4];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        T lz[8];
        for (int q = 0; q < 8; ++q) {
          T2 v = q < nz ? zin[((size_t)q * JB + r) * L + n] : mk<T2>(0, 0);
          lz[q] = e ? v.y : v.x;
        }
        T eta, Phi, U, V;
        if (mode == GM_ADJ_STEP) {
          T2 a0 = zin[((size_t)(nz + 0) * JB + r) * L + n], a1 = zin[((size_t)(nz + 1) * JB + r) * L + n];
          T2 a2 = zin[((size_t)(nz + 2) * JB + r) * L + n], a3 = zin[((size_t)(nz + 3) * JB + r) * L + n];
          eta = e ? a0.y : a0.x; Phi = e ? a1.y : a1.x; U = e ? a2.y : a2.x; V = e ? a3.y : a3.x;
        } else {
          size_t po = ((size_t)b * J + j) * I + 2 * n + e;
          eta = G.phys_in[0 * PS + po]; Phi = G.phys_in[2 * PS + po];
          U = G.phys_in[3 * PS + po]; V = G.phys_in[4 * PS + po];
        }
        pa.eval(eta, Phi, U, V, ihalf, sday[2 * n + e] * s, lz, lx[e], gacc);
      }
      if (mode == GM_ADJ_STEP) {
#pragma unroll
        for (int q = 0; q < 4; ++q) zout[((size_t)q * JB + r) * L + n] = mk<T2>(lx[0][q], lx[1][q]);
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
    block_add_grads<T>(gacc, sred, G.grad, B, b);
    if (mode == GM_ADJ_STEP) {
      // adjoint of x = Re(Y_0) + 2 Re sum_{m>=1} Y_m e^{i theta}:  lambda Y_m = c_m sum_i lambda x_i e^{-i theta}
      T2* res = cfft_batch<-1>(zout, zin, L, 4 * JB, g.twL);
      const int yf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
      const int rmap[5] = {0, -1, 1, 2, 3};
      for (int t = threadIdx.x; t < 5 * JB * (M + 1); t += blockDim.x) {
        int r = t % JB, k = (t / JB) % (M + 1), q = t / (JB * (M + 1));
        size_t o = ((size_t)k * B + b) * J + j0 + r;
        T2 v = G.lam[yf[q] * FS + o];
        if (rmap[q] >= 0) v = cadd(v, r2c_post<T2, T>(res + ((size_t)rmap[q] * JB + r) * L, L, k, g.twI, k == 0 ? (T)1 : (T)2));
        G.lamy[(size_t)q * FS + o] = v;
      }
      return;
    }
    // GM_ADJ_INIT batch 2: adjoint of the Fourier curr carries (fft(x/I)[:M+1]) of the ICs
    __syncthreads();
    const int cf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
    for (int t = threadIdx.x; t < 5 * JB * L; t += blockDim.x) {
      int k = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T2* y = G.lam + cf[f] * FS + (size_t)b * J + (j0 + r);
      bufA[(size_t)fr * L + k] = c2r_pre<T2, T>(y, B * J, M, L, k, g.twI, invI, invI * (T)0.5);
    }
    __syncthreads();
    T2* z2 = cfft_batch<+1>(bufA, bufB, L, 5 * JB, g.twL);
    for (int t = threadIdx.x; t < 5 * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      size_t po = f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      T2 v = z2[(size_t)fr * L + n];
      G.phys_out[po] += v.x;
      G.phys_out[po + 1] += v.y;
    }
    return;
  }

  if (mode == GM_ADJ_OUTPUT) {
    // ---------------------------------------------- seed: lambda of physical curr fields -> Fourier
    __syncthreads();
    const int nf = 5;
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * L + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch<-1>(bufA, bufB, L, nf * JB, g.twL);
    const int sf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
    for (int t = threadIdx.x; t < nf * JB * (M + 1); t += blockDim.x) {
      int r = t % JB, k = (t / JB) % (M + 1), f = t / (JB * (M + 1));
      T2 v = r2c_post<T2, T>(res + ((size_t)f * JB + r) * L, L, k, g.twI, k == 0 ? (T)1 : (T)2);
      G.lam[sf[f] * FS + ((size_t)k * B + b) * J + j0 + r] = v;
    }
    return;
  }

  if (mode == GM_FWD2) {
    // ------------------------------------------------ physical eta, delta -> Fourier
    __syncthreads();
    const int nf = 2;
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * L + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch<-1>(bufA, bufB, L, nf * JB, g.twL);
    for (int t = threadIdx.x; t < nf * JB * (M + 1); t += blockDim.x) {
      int r = t % JB, k = (t / JB) % (M + 1), f = t / (JB * (M + 1));
      T2 v = r2c_post<T2, T>(res + ((size_t)f * JB + r) * L, L, k, g.twI, invI);
      G.four[(f == 0 ? F_ETA : F_DELTA) * FS + ((size_t)k * B + b) * J + j0 + r] = v;
    }
    return;
  }

  if (mode == GM_INIT) {
    // ------------------------------------------------ physical ICs -> state
    // round 1: eta, delta, Phi, U, V  -> Fourier curr (+prev, mid) and residuals
    __syncthreads();
    const int nf = 5;
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      const T* x = G.phys_in + f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      bufA[(size_t)fr * L + n] = mk<T2>(x[0], x[1]);
    }
    __syncthreads();
    T2* res = cfft_batch<-1>(bufA, bufB, L, nf * JB, g.twL);
    T2* other = (res == bufA) ? bufB : bufA;
    const int sf[5] = {F_ETA, F_DELTA, F_PHI, F_U, F_V};
    // unpack into global and keep a copy of the truncated row in `other`
    for (int t = threadIdx.x; t < nf * JB * (M + 1); t += blockDim.x) {
      int r = t % JB, k = (t / JB) % (M + 1), f = t / (JB * (M + 1));
      T2 v = r2c_post<T2, T>(res + ((size_t)f * JB + r) * L, L, k, g.twI, invI);
      size_t o = ((size_t)k * B + b) * J + j0 + r;
      G.four[sf[f] * FS + o] = v;
      if (f < 3) {
        G.four[(f == 0 ? F_ETA_PREV : f == 1 ? F_DELTA_PREV : F_PHI_PREV) * FS + o] = v;
        G.four[(f == 0 ? F_ETA_MID : f == 1 ? F_DELTA_MID : F_PHI_MID) * FS + o] = v;
      }
      other[((size_t)f * JB + r) * (M + 1) + k] = v;
    }
    __syncthreads();
    // band-limited reconstruction -> residual = x - C2R(trunc FFT(x))
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int k = t % L, fr = t / L;
      res[(size_t)fr * L + k] = c2r_pre<T2, T>(other + (size_t)fr * (M + 1), 1, M, L, k, g.twI, (T)1, (T)1);
    }
    __syncthreads();
    T2* zr = cfft_batch<+1>(res, other, L, nf * JB, g.twL);
    for (int t = threadIdx.x; t < nf * JB * L; t += blockDim.x) {
      int n = t % L, fr = t / L, r = fr % JB, f = fr / JB;
      size_t po = f * PS + ((size_t)b * J + j0 + r) * I + 2 * n;
      const T* x = G.phys_in + po;
      T2 z = zr[(size_t)fr * L + n];
      G.resid[po] = x[0] - z.x;
      G.resid[po + 1] = x[1] - z.y;
    }
    __syncthreads();
    // round 2: nonlinear terms and forcing from the raw initial grids (model.py:723-732)
    double lrms = 0.0, lspin = 1e300;
    int nout = ph.forced ? 8 : 5;
    for (int t = threadIdx.x; t < JB * L; t += blockDim.x) {
      int n = t % L, r = t / L, j = j0 + r;
      size_t po = ((size_t)b * J + j) * I + 2 * n;
      T ihalf = (T)(1.0 / (2.0 * g.onemu2[j]));
      T s = (T)sqrt(g.onemu2[j]);
      T outs[2][8];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        T eta = G.phys_in[0 * PS + po + e], Phi = G.phys_in[2 * PS + po + e];
        T U = G.phys_in[3 * PS + po + e], V = G.phys_in[4 * PS + po + e];
        ph.eval(eta, Phi, U, V, ihalf, sday[2 * n + e] * s, outs[e]);
        if (cfg.diagnostics) {
          double Ud = U, Vd = V;
          lrms += g.area[j] * (Ud * Ud + Vd * Vd);
          lspin = fmin(lspin, sqrt(Ud * Ud + Vd * Vd));
        }
      }
      for (int q = 0; q < nout; ++q) bufA[((size_t)q * JB + r) * L + n] = mk<T2>(outs[0][q], outs[1][q]);
    }
    if (cfg.diagnostics) {
      for (int o = 16; o > 0; o >>= 1) {
        lrms += __shfl_down_sync(0xffffffffu, lrms, o);
        lspin = fmin(lspin, __shfl_down_sync(0xffffffffu, lspin, o));
      }
      if ((threadIdx.x & 31) == 0) { atomicAdd(&sred[0], lrms); atomic_min_d(&sred[1], lspin); }
    }
    __syncthreads();
    if (cfg.diagnostics && threadIdx.x == 0) {
      double* d0 = G.diag;
      atomicAdd(&d0[D_RMS2 * B + b], sred[0]);
      atomic_min_d(&d0[D_SPIN * B + b], sred[1]);
    }
    T2* res2 = cfft_batch<-1>(bufA, bufB, L, nout * JB, g.twL);
    for (int t = threadIdx.x; t < nout * JB * (M + 1); t += blockDim.x) {
      int r = t % JB, k = (t / JB) % (M + 1), q = t / (JB * (M + 1));
      T2 v = r2c_post<T2, T>(res2 + ((size_t)q * JB + r) * L, L, k, g.twI, invI);
      G.four[(F_A + q) * FS + ((size_t)k * B + b) * J + j0 + r] = v;
    }
    return;
  }
}

void grid_set_attributes() {
  cudaFuncSetAttribute(k_grid<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(k_grid<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename T>
cudaError_t launch_grid(const GridLaunch<T>& L, int nblocks, size_t smem, cudaStream_t s) {
  k_grid<T><<<nblocks, 256, smem, s>>>(L);
  return cudaGetLastError();
}
template cudaError_t launch_grid<double>(const GridLaunch<double>&, int, size_t, cudaStream_t);
template cudaError_t launch_grid<float>(const GridLaunch<float>&, int, size_t, cudaStream_t);

}  // namespace swp
