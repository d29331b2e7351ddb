// Shared definitions for the SWAMPE GB300 time-stepping kernels.
//
// Layout conventions (all device memory is owned by the caller):
//   * Fourier field  : complex[M+1][B][J]   (m slowest, latitude j fastest), per field
//   * physical field : real[B][J][I]
//   * per-member scalar parameters: double[NPAR][B]
// The complex element type is T2 (double2 or float2), real parts first.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace swp {

// ---------------------------------------------------------------- params ---
enum ParamIndex {
  P_DT = 0, P_A, P_OMEGA, P_PHIBAR, P_TAURAD, P_TAUDRAG, P_DPHIEQ, P_K6, P_K6PHI, P_ALPHA,
  P_SIALPHA,  // implicit weight of the semi-implicit scheme (RunFlags.si_alpha)
  P_WALPHA,   // Williams weight of the RAW filter (RunFlags.williams_alpha)
  NPAR
};

// Fourier-space state fields, in the order used by the kernels.
enum FourierField {
  F_ETA_PREV = 0, F_ETA, F_DELTA_PREV, F_DELTA, F_PHI_PREV, F_PHI, F_U, F_V,
  F_A, F_B, F_C, F_D, F_E, F_PHIF, F_F, F_G, F_ETA_MID, F_DELTA_MID, F_PHI_MID,
  NFOURIER
};
// The semi-implicit scheme reads the filtered lineage (*_MID) as its n-1 base
// and never the unfiltered prev carries; their slots hold its lagged
// momentum-forcing remainders (model.py:775-792, 1135-1143).
constexpr int F_RU_LAG = F_ETA_PREV;
constexpr int F_RV_LAG = F_DELTA_PREV;

// Physical residual fields (initial condition minus its band-limited part).
enum ResidualField { R_ETA = 0, R_DELTA, R_PHI, R_U, R_V, NRESID };

template <typename T> struct cplx;
template <> struct cplx<double> { typedef double2 type; };
template <> struct cplx<float> { typedef float2 type; };

// Scalar type of a complex vector type.  mk takes its arguments in that type:
// a double signature would round-trip every float through FP64 conversions.
template <typename T2> struct scalar_of;
template <> struct scalar_of<double2> { typedef double type; };
template <> struct scalar_of<float2> { typedef float type; };
template <typename T2>
__device__ __forceinline__ T2 mk(typename scalar_of<T2>::type r, typename scalar_of<T2>::type i) {
  T2 z; z.x = r; z.y = i; return z;
}
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { T2 z; z.x = a.x + b.x; z.y = a.y + b.y; return z; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { T2 z; z.x = a.x - b.x; z.y = a.y - b.y; return z; }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 z; z.x = a.x * b.x - a.y * b.y; z.y = a.x * b.y + a.y * b.x; return z;
}
// a * conj(b)
template <typename T2> __device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
  T2 z; z.x = a.x * b.x + a.y * b.y; z.y = a.y * b.x - a.x * b.y; return z;
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { a.y = -a.y; return a; }

// 16-byte global accesses of consecutive latitude rows: two complex values in
// FP32, one in FP64 (Fourier fields keep the latitude fastest, so rows j, j+1
// of one (m, member) are adjacent; the pointer is 16-byte aligned).  The
// kernels are bound by the number of memory instructions in flight per SM
// rather than by bytes, so each access moves 16 bytes.
template <typename T2> struct Rows16 { static constexpr int N = 16 / (int)sizeof(T2); };
__device__ __forceinline__ void ld_rows16(const float2* p, float2 (&v)[2]) {
  const float4 w = *(const float4*)p;
  v[0] = make_float2(w.x, w.y);
  v[1] = make_float2(w.z, w.w);
}
__device__ __forceinline__ void ld_rows16(const double2* p, double2 (&v)[1]) { v[0] = *p; }
__device__ __forceinline__ void st_rows16(float2* p, const float2 (&v)[2]) {
  *(float4*)p = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
}
__device__ __forceinline__ void st_rows16(double2* p, const double2 (&v)[1]) { *p = v[0]; }
template <typename T2> __device__ __forceinline__ T2 cscale(T2 a, typename scalar_of<T2>::type s) {
  a.x *= s; a.y *= s; return a;
}
// multiply by +i (SIGN>0) or -i (SIGN<0)
template <int SIGN, typename T2> __device__ __forceinline__ T2 cmul_i(T2 a) {
  T2 z; if (SIGN > 0) { z.x = -a.y; z.y = a.x; } else { z.x = a.y; z.y = -a.x; } return z;
}

// ------------------------------------------------------------ small DFTs ---
// Forward (SIGN=-1) or inverse (SIGN=+1) DFT of R points held in registers.
template <int SIGN, typename T2> __device__ __forceinline__ void dft2(T2* v) {
  T2 a = v[0], b = v[1]; v[0] = cadd(a, b); v[1] = csub(a, b);
}

template <int SIGN, typename T2> __device__ __forceinline__ void dft3(T2* v) {
  typedef decltype(v[0].x) T;
  const T c = (T)-0.5;
  const T s = (T)(SIGN * 0.86602540378443864676);  // sin(+-2pi/3)
  T2 a = cadd(v[1], v[2]), b = csub(v[1], v[2]);
  T2 base = mk<T2>(v[0].x + c * a.x, v[0].y + c * a.y);
  T2 ib = mk<T2>(-s * b.y, s * b.x);  // i*s*b
  v[0] = cadd(v[0], a);
  v[1] = cadd(base, ib);
  v[2] = csub(base, ib);
}

template <int SIGN, typename T2> __device__ __forceinline__ void dft4(T2* v) {
  T2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  T2 t2 = cadd(v[1], v[3]), t3 = cmul_i<SIGN>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3); v[3] = csub(t1, t3);
}

template <int SIGN, typename T2> __device__ __forceinline__ void dft5(T2* v) {
  typedef decltype(v[0].x) T;
  const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
  const T s1 = (T)(SIGN * 0.95105651629515357212), s2 = (T)(SIGN * 0.58778525229247312917);
  T2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
  T2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
  T2 x0 = v[0];
  T2 r1 = mk<T2>(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
  T2 r2 = mk<T2>(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
  // i*(s1 b1 + s2 b2) and i*(s2 b1 - s1 b2)
  T2 q1 = mk<T2>(-(s1 * b1.y + s2 * b2.y), s1 * b1.x + s2 * b2.x);
  T2 q2 = mk<T2>(-(s2 * b1.y - s1 * b2.y), s2 * b1.x - s1 * b2.x);
  v[0] = mk<T2>(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
  v[1] = cadd(r1, q1); v[4] = csub(r1, q1);
  v[2] = cadd(r2, q2); v[3] = csub(r2, q2);
}

template <int SIGN, typename T2> __device__ __forceinline__ void dft8(T2* v) {
  typedef decltype(v[0].x) T;
  T2 e[4] = {v[0], v[2], v[4], v[6]};
  T2 o[4] = {v[1], v[3], v[5], v[7]};
  dft4<SIGN>(e); dft4<SIGN>(o);
  const T h = (T)0.70710678118654752440;
  // w8^k = exp(SIGN * i * 2pi k / 8)
  T2 w1o = mk<T2>(h * (o[1].x - SIGN * o[1].y), h * (o[1].y + SIGN * o[1].x));
  T2 w2o = cmul_i<SIGN>(o[2]);
  T2 w3o = mk<T2>(h * (-o[3].x - SIGN * o[3].y), h * (-o[3].y + SIGN * o[3].x));
  v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], w1o);  v[5] = csub(e[1], w1o);
  v[2] = cadd(e[2], w2o);  v[6] = csub(e[2], w2o);
  v[3] = cadd(e[3], w3o);  v[7] = csub(e[3], w3o);
}

template <int R, int SIGN, typename T2> __device__ __forceinline__ void dftR(T2* v) {
  if (R == 2) dft2<SIGN>(v);
  else if (R == 3) dft3<SIGN>(v);
  else if (R == 4) dft4<SIGN>(v);
  else if (R == 5) dft5<SIGN>(v);
  else dft8<SIGN>(v);
}

// One Stockham autosort pass (radix R) over `ntr` transforms of length L held
// in shared memory with stride `ls` (transform t at in + t*ls; ls = L+1 keeps
// the transforms of a warp on different banks).  tw[k] = exp(-2 pi i k / L).
template <int R, int SIGN, typename T2>
__device__ __forceinline__ void stockham_pass(const T2* __restrict__ in, T2* __restrict__ out,
                                              int L, int ls, int ns, int ntr, const T2* __restrict__ tw) {
  const int per = L / R;
  const int tasks = ntr * per;
  const int twstride = L / (ns * R);
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    int t = task / per, j = task - t * per;
    const T2* src = in + t * ls;
    T2* dst = out + t * ls;
    int jm = j % ns;
    T2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * per];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      int k = jm * r * twstride;  // < L
      T2 w = tw[k];
      v[r] = (SIGN < 0) ? cmul(v[r], w) : cmulc(v[r], w);
    }
    dftR<R, SIGN>(v);
    int idx = (j / ns) * ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[idx + r * ns] = v[r];
  }
}

// Complex FFT of `ntr` length-L transforms (stride ls) held in smem buffer a
// (b is scratch).  Returns the buffer holding the result.  L in {64, 96, 160}.
template <int SIGN, typename T2>
__device__ T2* cfft_batch(T2* a, T2* b, int L, int ls, int ntr, const T2* tw) {
  if (L == 64) {
    stockham_pass<8, SIGN>(a, b, L, ls, 1, ntr, tw); __syncthreads();
    stockham_pass<8, SIGN>(b, a, L, ls, 8, ntr, tw); __syncthreads();
    return a;
  } else if (L == 96) {
    stockham_pass<8, SIGN>(a, b, L, ls, 1, ntr, tw); __syncthreads();
    stockham_pass<4, SIGN>(b, a, L, ls, 8, ntr, tw); __syncthreads();
    stockham_pass<3, SIGN>(a, b, L, ls, 32, ntr, tw); __syncthreads();
    return b;
  } else {  // 160
    stockham_pass<8, SIGN>(a, b, L, ls, 1, ntr, tw); __syncthreads();
    stockham_pass<4, SIGN>(b, a, L, ls, 8, ntr, tw); __syncthreads();
    stockham_pass<5, SIGN>(a, b, L, ls, 32, ntr, tw); __syncthreads();
    return b;
  }
}

// n / d for 0 <= n < 2^16 and 2 <= d <= 256 by one multiply-high (exact in
// that range: the rounding error of the reciprocal stays below 1/d).
struct FastDiv {
  uint32_t m;
  __device__ __forceinline__ explicit FastDiv(int d) : m(0xFFFFFFFFu / (uint32_t)d + 1u) {}
  __device__ __forceinline__ int operator()(int n) const { return (int)__umulhi((uint32_t)n, m); }
};

// Compile-time-length variant of the above (ls = L + 1).  Lanes take the same
// butterfly of consecutive transforms (transform index fastest): with the odd
// stride L + 1 every load and store of a pass is free of bank conflicts once a
// half-warp spans 16 transforms.  ntr >= 2.
template <int R, int SIGN, int L, int NS, typename T2>
__device__ __forceinline__ void stockham_pass_c(const T2* __restrict__ in, T2* __restrict__ out, int ntr,
                                                const T2* __restrict__ tw) {
  constexpr int LS = L + 1, PER = L / R, TWS = L / (NS * R);
  const int tasks = ntr * PER;
  const FastDiv divt(ntr);
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int j = divt(task), t = task - j * ntr;
    const T2* src = in + t * LS;
    T2* dst = out + t * LS;
    const int jm = j % NS;
    T2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * PER];
    if (NS > 1) {  // the first pass has no twiddles
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const T2 w = tw[jm * r * TWS];
        v[r] = (SIGN < 0) ? cmul(v[r], w) : cmulc(v[r], w);
      }
    }
    dftR<R, SIGN>(v);
    const int idx = (j / NS) * NS * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[idx + r * NS] = v[r];
  }
}

template <int SIGN, int L, typename T2>
__device__ __forceinline__ T2* cfft_batch_c(T2* a, T2* b, int ntr, const T2* tw) {
  static_assert(L == 64 || L == 96 || L == 160, "transform length");
  if (L == 64) {
    stockham_pass_c<8, SIGN, L, 1>(a, b, ntr, tw); __syncthreads();
    stockham_pass_c<8, SIGN, L, 8>(b, a, ntr, tw); __syncthreads();
    return a;
  } else if (L == 96) {
    stockham_pass_c<8, SIGN, L, 1>(a, b, ntr, tw); __syncthreads();
    stockham_pass_c<4, SIGN, L, 8>(b, a, ntr, tw); __syncthreads();
    stockham_pass_c<3, SIGN, L, 32>(a, b, ntr, tw); __syncthreads();
    return b;
  } else {
    stockham_pass_c<8, SIGN, L, 1>(a, b, ntr, tw); __syncthreads();
    stockham_pass_c<4, SIGN, L, 8>(b, a, ntr, tw); __syncthreads();
    stockham_pass_c<5, SIGN, L, 32>(a, b, ntr, tw); __syncthreads();
    return b;
  }
}

// Passes 2.. of cfft_batch_c after a first radix-8 pass (NS = 1) that left its
// output in `a`.  Returns the buffer holding the result.
template <int SIGN, int L, typename T2>
__device__ __forceinline__ T2* cfft_rest_c(T2* a, T2* b, int ntr, const T2* tw) {
  static_assert(L == 64 || L == 96 || L == 160, "transform length");
  if (L == 64) {
    stockham_pass_c<8, SIGN, L, 8>(a, b, ntr, tw); __syncthreads();
    return b;
  } else if (L == 96) {
    stockham_pass_c<4, SIGN, L, 8>(a, b, ntr, tw); __syncthreads();
    stockham_pass_c<3, SIGN, L, 32>(b, a, ntr, tw); __syncthreads();
    return a;
  } else {
    stockham_pass_c<4, SIGN, L, 8>(a, b, ntr, tw); __syncthreads();
    stockham_pass_c<5, SIGN, L, 32>(b, a, ntr, tw); __syncthreads();
    return a;
  }
}

// Gauss grid of each supported truncation (the reference's M -> (J, I) table,
// spectral_transform.py / model.py: 42 -> 64 x 128, 63 -> 96 x 192, 106 -> 160 x 320).
__host__ __device__ constexpr int trunc_J(int M) { return M == 42 ? 64 : M == 63 ? 96 : 160; }
__host__ __device__ constexpr int trunc_I(int M) { return 2 * trunc_J(M); }

// ------------------------------------------------------------- descriptors ---
// Geometry for one truncation, built on the device in FP64 (geometry.cu) and
// rounded to the compute type.  Basis blocks are packed per zonal wavenumber m
// and split by the parity of (n - m):
//   fwd layout  [par][j'][c]  (j' = 0..J/2-1 southern nodes, n = m + par + 2c)
//   inv layout  [par][c][j']
// boff[m] is the element offset of block m (same for all four bases).
template <typename T>
struct Geom {
  int M, J, I, L;          // truncation, latitudes, longitudes, L = I/2
  const double* mu;        // [J]
  const double* w;         // [J]
  const double* onemu2;    // [J]  1 - mu^2
  const double* area;      // [J]  RMS-wind area weight / cos^2(phi)
  const int* boff;         // [M+2]
  const T* Pw_f; const T* Hw_f;   // weighted basis, fwd layout
  const T* P_f;  const T* H_f;    // unweighted basis, fwd layout (adjoint of inverse)
  const T* P_i;  const T* H_i;    // unweighted basis, inv layout
  const T* Pw_i; const T* Hw_i;   // weighted basis, inv layout (adjoint of forward)
  const typename cplx<T>::type* twL;  // [L]   exp(-2 pi i k / L)
  const typename cplx<T>::type* twI;  // [L+1] exp(-2 pi i k / I)
  const T* dayc;           // [I]  dayside-mask * cos(lambda)
  const T* ihalf;          // [J]  1 / (2 (1 - mu^2))
  const T* coslat;         // [J]  sqrt(1 - mu^2)
};

// Step configuration shared by a launch.
struct StepCfg {
  int scheme;      // 0 = modified Euler, 1 = explicit, 2 = semi-implicit
  int forcflag;
  int diffflag;
  int test;        // 0 = forced (test None), 1, 2
  int ra_mode;     // 0 = leave RA mid, 1 = mid <- curr, 2 = Robert-Asselin update
  int write_prev;  // copy old curr into the Fourier prev carry
  int diagnostics; // blow-up gate + reductions
  double blowup;   // RMS threshold
  int step;        // scan-step index (row of the diagnostic arrays)
  int incremental; // advance a band-limited state by increments (FP32 path)
  int lam_fg_tied; // adjoint sweep: lambda_F = lambda_B, lambda_G = -lambda_A hold (forced)
  int raw;         // Robert-Asselin-Williams filter: the new level moves too
  int si_relax;    // semi-implicit: relaxation and drag implicit (forcflag, test None)
  int si_lag_init; // semi-implicit first step: lagged remainder from the current state
  int tl_coef;     // tangent-linear step: differentiate the coefficient tables too
  int tl_filter;   // primal step of a tangent run: add the filter weights' tangents times the
                   // displacement to the tangent carries (SpecGroup four_t, dw)
  int adj_zeroed;  // modified-Euler adjoint sweep after its first step: the adjoint of U, V and
                   // of the prev / mid carries is already zero (an earlier step of the sweep
                   // wrote it), so the step neither reads nor rewrites it
};

// Programmatic dependent launch.  The step kernels are launched with the
// programmatic-serialization attribute (launch_pdl), so that a kernel's CTAs
// can be scheduled while its predecessor in the stream drains its last wave.
// Every such kernel lets its own dependent launch at once and then waits, before
// its first access to global memory that another kernel writes, until the
// predecessor has completed and its writes are visible.  Launched without the
// attribute, both instructions return at once.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
  pdl_trigger();
  pdl_wait();
}

}  // namespace swp
