// Building blocks of the grid kernels (grid.cu): the grid-space physics and
// its adjoint and tangent, the half-length C2R / R2C bin maps, double atomics
// and the group lookup of a launch.
#pragma once
#include <float.h>
#include "swp_internal.h"

namespace swp {

// x / pts on the FP32 path as x * (correctly rounded 1/pts): one reciprocal
// per point instead of IEEE divisions (within 1 ulp of the quotient); the FP64
// path divides exactly.
__device__ __forceinline__ float div_pts(float x, float inv, float) { return x * inv; }
__device__ __forceinline__ double div_pts(double x, double, double pts) { return x / pts; }
__device__ __forceinline__ float recip_pts(float pts) { return __frcp_rn(pts); }
__device__ __forceinline__ double recip_pts(double) { return 0.0; }

template <typename T> __device__ __forceinline__ T tiny_val();
template <> __device__ __forceinline__ double tiny_val<double>() { return DBL_MIN; }
template <> __device__ __forceinline__ float tiny_val<float>() { return FLT_MIN; }

template <typename T>
__device__ __forceinline__ const GridGroup<T>& pick_ggroup(const GridLaunch<T>& L, int& idx) {
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  idx = blockIdx.x - L.prefix[gi];
  return L.grp[gi];
}

// Half-length spectrum Z_k (k < L) of the C2R transform
//   x_i = Re(Y_0) + 2 Re sum_{m=1..M} Y_m e^{2 pi i m i / I},   x_{2n} + i x_{2n+1} = sum_k Z_k e^{2 pi i k n / L}
// from the truncated row y[m * ys], m = 0..M.  scale0 / scale multiply Y_0 / Y_m.
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

// Bin k (0..M) of the R2C transform from the half-length spectrum Z (after the
// forward FFT of x_{2n} + i x_{2n+1}), times `scale`.
template <typename T2, typename T>
__device__ __forceinline__ T2 r2c_post(const T2* Z, int L, int k, const T2* twI, T scale) {
  T2 zk = Z[k], zl = cconj(Z[(L - k) % L]);
  T2 e = cscale(cadd(zk, zl), (T)0.5);
  T2 d = csub(zk, zl);
  T2 o; o.x = (T)0.5 * d.y; o.y = (T)-0.5 * d.x;  // d / (2i)
  return cscale(cadd(e, cmul(o, twI[k])), scale);
}

// Asynchronous global -> shared copy of one element (8 or 16 bytes, aligned to
// its size); the issuing thread completes its copies with cp_async_wait_all.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  static_assert(BYTES == 8 || BYTES == 16, "cp.async copies 8 or 16 bytes here");
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

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
  __device__ __forceinline__ void eval(T eta, T Phi, T U, T V, T ihalf, T day_s, T* out) const {
    // ABCDE_init (initial_conditions.py:499-503)
    out[0] = U * eta; out[1] = V * eta; out[2] = U * Phi; out[3] = V * Phi;
    out[4] = (U * U + V * V) * ihalf;
    if (forced) {
      T Phieq = Pb + DPe * day_s;                        // forcing.py:55-60
      T Q = itr * (Phieq - (Phi + Pb));                  // forcing.py:94
      T Qc = Q < (T)0 ? (T)0 : Q;                        // forcing.py:133
      T pt = Phi + Pb;
      T pts = fabs(pt) > (T)0 ? pt : tiny_val<T>();     // forcing.py:139-140
      T r = div_pts(Qc, recip_pts(pts), pts);
      T Ru = -U * r, Rv = -V * r;
      out[5] = Q;
      out[6] = nodrag ? Ru : Ru - U * itd;               // forcing.py:143-153
      out[7] = nodrag ? Rv : Rv - V * itd;
    } else {
      out[5] = out[6] = out[7] = (T)0;
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
  __device__ __forceinline__ void eval(T eta, T Phi, T U, T V, T ihalf, T day_s, const T* lz, T* lx,
                                       T* gacc) const {
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
      const T ipts = recip_pts(pts);
      T r = div_pts(Qc, ipts, pts);
      T lF = lz[6], lG = lz[7];
      T lr = -U * lF - V * lG;
      T itdd = nodrag ? (T)0 : itd;
      lU += lF * (-r - itdd);
      lV += lG * (-r - itdd);
      T lQc = div_pts(lr, ipts, pts);
      T lpts = div_pts(-lr * r, ipts, pts);
      T lQ = lz[5] + (pos ? lQc : (T)0);
      lPhi += -itr * lQ + lpts;
      // per-thread partial sums in the compute type (two points per thread);
      // the block and global reductions run in FP64
      gacc[G_TAURAD] += lQ * (-Q * itr);
      if (!nodrag) gacc[G_TAUDRAG] += (lF * U + lG * V) * itd * itd;
      gacc[G_DPHIEQ] += lQ * itr * day_s;
      gacc[G_PHIBAR] += lpts;
    }
    lx[0] = leta; lx[1] = lPhi; lx[2] = lU; lx[3] = lV;
  }
};

// Tangent of Physics::eval (forward mode): x = (eta, Phi, U, V) with tangent
// dx, parameter tangents dp = d(taurad, taudrag, DPhieq, Phibar).  Same
// branch conventions as the adjoint: the clamp passes no tangent where Q < 0,
// Phieq's Phibar cancels in Q, taudrag = -1 has no drag term.
template <typename T>
struct PhysicsTL {
  T Pb, itr, itd, DPe;
  bool nodrag, forced;
  __device__ __forceinline__ void eval(T eta, T Phi, T U, T V, T deta, T dPhi, T dU, T dV, T ihalf, T day_s,
                                       const T* dp, T* out) const {
    out[0] = dU * eta + U * deta;
    out[1] = dV * eta + V * deta;
    out[2] = dU * Phi + U * dPhi;
    out[3] = dV * Phi + V * dPhi;
    out[4] = (T)2 * (U * dU + V * dV) * ihalf;
    if (forced) {
      T Phieq = Pb + DPe * day_s;
      T Q = itr * (Phieq - (Phi + Pb));
      // dQ = -itr dPhi - Q itr dtaurad + itr day_s dDPhieq
      T dQ = itr * (day_s * dp[G_DPHIEQ] - dPhi) - Q * itr * dp[G_TAURAD];
      bool pos = !(Q < (T)0);
      T Qc = pos ? Q : (T)0, dQc = pos ? dQ : (T)0;
      T pt = Phi + Pb;
      T pts = fabs(pt) > (T)0 ? pt : tiny_val<T>();
      const T ipts = recip_pts(pts);
      T r = div_pts(Qc, ipts, pts);
      T dr = div_pts(dQc - r * (dPhi + dp[G_PHIBAR]), ipts, pts);
      T dRu = -(dU * r + U * dr), dRv = -(dV * r + V * dr);
      out[5] = dQ;
      if (nodrag) {
        out[6] = dRu;
        out[7] = dRv;
      } else {
        // d(U / taudrag) = dU itd - U itd^2 dtaudrag
        const T ditd = itd * itd * dp[G_TAUDRAG];
        out[6] = dRu - dU * itd + U * ditd;
        out[7] = dRv - dV * itd + V * ditd;
      }
    } else {
      out[5] = out[6] = out[7] = (T)0;
    }
  }
};

}  // namespace swp
