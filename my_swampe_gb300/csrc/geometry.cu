// Static geometry for one spectral truncation, computed on the GPU in FP64.
//
// Replaces the host-side SciPy set-up of the reference:
//   spectral_transform.py:80-114  gauss_legendre  (roots_legendre)
//   spectral_transform.py:219-287 PmnHmn          (assoc_legendre_p_all, scaling, odd-m flip)
//   spectral_transform.py:351-367 weighted_legendre_basis
//   time_stepping.py:537-576      RMS_winds area weights
//   forcing.py:14-62              dayside mask * cos(lambda)
// The basis is the fully normalised associated Legendre function without the
// Condon-Shortley phase, which is what the reference's scaling table plus
// odd-m sign flip produce.  It is evaluated with the standard three-term
// recurrence in n, and H = (1 - mu^2) dP/dmu from the derivative identity
//   (1-x^2) dPbar_n^m/dx = -n x Pbar_n^m + sqrt((2n+1)/(2n-1) (n^2-m^2)) Pbar_{n-1}^m.
#include <cmath>
#include "swp_internal.h"

namespace swp {

// One thread per southern node j' < J/2: Newton iteration on P_J, mirrored.
__global__ void k_gauss_nodes(int J, double* mu, double* w, int* err) {
  int jh = J / 2;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= jh) return;
  double x = -cospi((j + 0.75) / (J + 0.5));
  double dp = 1.0;
  bool converged = false;
  for (int it = 0; it < 100; ++it) {  // bounded: converges in < 10 steps
    double p0 = 1.0, p1 = x;
    for (int n = 2; n <= J; ++n) {
      double p2 = ((2.0 * n - 1.0) * x * p1 - (n - 1.0) * p0) / n;
      p0 = p1; p1 = p2;
    }
    dp = J * (x * p1 - p0) / (x * x - 1.0);
    double dx = p1 / dp;
    x -= dx;
    if (fabs(dx) <= 4e-16 * fabs(x) + 1e-300) { converged = true; break; }
  }
  if (!converged) {
    // one more Newton update at the last iterate; fail only if it is not at round-off level
    double p0 = 1.0, p1 = x;
    for (int n = 2; n <= J; ++n) {
      double p2 = ((2.0 * n - 1.0) * x * p1 - (n - 1.0) * p0) / n;
      p0 = p1; p1 = p2;
    }
    double d = J * (x * p1 - p0) / (x * x - 1.0);
    if (fabs(p1 / d) > 1e-14) atomicExch(err, 1);
  }
  // weight at the exact root x* = x - delta (delta = P_J/P_J', below one ulp):
  //   w = 2 / ((1-x^2) P_J'^2),  d ln w / dx = 2x/(1-x^2) - 2 P_J''/P_J',
  //   P_J'' = (2x P_J' - J(J+1) P_J) / (1-x^2)   (Legendre's equation)
  // The first-order correction removes the ~1e3..1e4 amplification of the
  // last-ulp root error near the poles.
  double p0 = 1.0, p1 = x;
  for (int n = 2; n <= J; ++n) {
    double p2 = ((2.0 * n - 1.0) * x * p1 - (n - 1.0) * p0) / n;
    p0 = p1; p1 = p2;
  }
  double omx2 = (1.0 - x) * (1.0 + x);
  dp = J * (p0 - x * p1) / omx2;
  double wt = 2.0 / (omx2 * dp * dp);
  double delta = p1 / dp;
  double d2 = (2.0 * x * dp - (double)J * (J + 1.0) * p1) / omx2;
  wt *= 1.0 - delta * (2.0 * x / omx2 - 2.0 * d2 / dp);
  mu[j] = x;
  mu[J - 1 - j] = -x;
  w[j] = wt;
  w[J - 1 - j] = wt;
}

// Per-latitude constants that need neighbouring nodes (RMS-wind weights).
__global__ void k_lat_consts(int J, int I, const double* mu, double* onemu2, double* area, double* ihalf64,
                             double* coslat64, float* ihalf32, float* coslat32) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= J) return;
  onemu2[j] = 1.0 - mu[j] * mu[j];
  // 1 / (2 (1 - mu^2)) of the kinetic-energy term E (initial_conditions.py:499-503)
  // and cos(phi) = sqrt(1 - mu^2) of the dayside forcing (forcing.py:55-60),
  // per latitude in both compute types
  const double ih = 1.0 / (2.0 * onemu2[j]), cl = sqrt(onemu2[j]);
  ihalf64[j] = ih;
  coslat64[j] = cl;
  ihalf32[j] = (float)ih;
  coslat32[j] = (float)cl;
  // time_stepping.py:568-576: area_comp = a^2 sin(phi+pi/2)^2 dphi dlambda,
  // integrand (U/cos phi)^2 + (V/cos phi)^2, normalised by 4 pi a^2.
  double phi = asin(mu[j]);
  double dphi = asin(mu[2]) - asin(mu[1]);
  double lam1 = -M_PI + 2.0 * M_PI * 1.0 / I, lam2 = -M_PI + 2.0 * M_PI * 2.0 / I;
  double dlam = lam2 - lam1;
  double s = sin(phi + M_PI / 2.0);
  double c = cos(phi);
  area[j] = (s * s * dphi * dlam) / (c * c) / (4.0 * M_PI);
}

// One thread per (m, j'): recurrence in n, written into the packed layouts.
__global__ void k_basis(int M, int J, const double* mu, const double* w, const int* boff, const double* damage,
                        double* Pw_f, double* Hw_f, double* P_f, double* H_f,
                        double* P_i, double* H_i, double* Pw_i, double* Hw_i,
                        float* Pw_f32, float* Hw_f32, float* P_f32, float* H_f32,
                        float* P_i32, float* H_i32, float* Pw_i32, float* Hw_i32) {
  int jh = J / 2;
  int m = blockIdx.x;
  int j = threadIdx.x + blockIdx.y * blockDim.x;
  if (m > M || j >= jh) return;
  int N = M;
  int cnt = N + 1 - m;
  int C0 = (cnt + 1) / 2;
  int base = boff[m];
  double x = mu[j];
  double s = sqrt(1.0 - x * x);
  double wt = w[j];
  // Pbar_m^m without Condon-Shortley phase
  double pmm = sqrt(0.5);
  for (int k = 1; k <= m; ++k) pmm *= sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
  double pm2 = 0.0, pm1 = pmm;  // P_{n-2}, P_{n-1}
  for (int n = m; n <= N; ++n) {
    double P;
    if (n == m) P = pmm;
    else if (n == m + 1) P = sqrt(2.0 * m + 3.0) * x * pmm;
    else {
      double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
      double b = sqrt((((double)(n - 1) * (n - 1)) - (double)m * m) / (4.0 * (n - 1) * (n - 1) - 1.0));
      P = a * (x * pm1 - b * pm2);
    }
    double Pprev = (n == m) ? 0.0 : pm1;
    double H = -n * x * P;
    if (n > m) H += sqrt((2.0 * n + 1.0) / (2.0 * n - 1.0) * ((double)n * n - (double)m * m)) * Pprev;
    if (n > m) { pm2 = pm1; pm1 = P; }
    double dmg = damage[m * (N + 1) + n];
    P *= dmg;
    H *= dmg;
    int k = n - m, par = k & 1, c = k >> 1;
    int poff = par ? jh * C0 : 0;
    int Cp = par ? cnt / 2 : C0;
    int fi = base + poff + j * Cp + c;   // fwd [par][j'][c]
    int ii = base + poff + c * jh + j;   // inv [par][c][j']
    Pw_f[fi] = wt * P; Hw_f[fi] = wt * H; P_f[fi] = P; H_f[fi] = H;
    P_i[ii] = P; H_i[ii] = H; Pw_i[ii] = wt * P; Hw_i[ii] = wt * H;
    Pw_f32[fi] = (float)(wt * P); Hw_f32[fi] = (float)(wt * H); P_f32[fi] = (float)P; H_f32[fi] = (float)H;
    P_i32[ii] = (float)P; H_i32[ii] = (float)H; Pw_i32[ii] = (float)(wt * P); Hw_i32[ii] = (float)(wt * H);
  }
}

// Dense (J, M+1, N+1) copies for the Static-compatible host view.
__global__ void k_basis_dense(int M, int J, const int* boff, const double* P_f, const double* H_f,
                              double* Pd, double* Hd) {
  int jh = J / 2;
  int m = blockIdx.x;
  int N = M;
  for (int idx = threadIdx.x; idx < J * (N + 1); idx += blockDim.x) {
    int j = idx / (N + 1), n = idx % (N + 1);
    double p = 0.0, h = 0.0;
    if (n >= m) {
      int cnt = N + 1 - m, C0 = (cnt + 1) / 2;
      int k = n - m, par = k & 1, c = k >> 1;
      int jj = j < jh ? j : J - 1 - j;
      int Cp = par ? cnt / 2 : C0;
      int fi = boff[m] + (par ? jh * C0 : 0) + jj * Cp + c;
      p = P_f[fi];
      h = H_f[fi];
      if (j >= jh) {  // mirror: P(-mu) = (-1)^(n-m) P(mu), H(-mu) = -(-1)^(n-m) H(mu)
        double sgn = par ? -1.0 : 1.0;
        p *= sgn;
        h *= -sgn;
      }
    }
    size_t o = ((size_t)j * (M + 1) + m) * (N + 1) + n;
    Pd[o] = p;
    Hd[o] = h;
  }
}

__global__ void k_twiddles(int I, double2* twL64, double2* twI64, float2* twL32, float2* twI32,
                           double* dayc64, float* dayc32) {
  int L = I / 2;
  for (int k = threadIdx.x + blockIdx.x * blockDim.x; k <= I; k += blockDim.x * gridDim.x) {
    if (k < L) {
      double s, c;
      sincospi(-2.0 * k / L, &s, &c);
      twL64[k] = make_double2(c, s);
      twL32[k] = make_float2((float)c, (float)s);
    }
    if (k <= L) {
      double s, c;
      sincospi(-2.0 * k / I, &s, &c);
      twI64[k] = make_double2(c, s);
      twI32[k] = make_float2((float)c, (float)s);
    }
    if (k < I) {
      // lambda_i = -pi + 2 pi i / I; strict dayside -pi/2 < lambda < pi/2 <=> I/4 < i < 3I/4
      bool day = (4 * k > I) && (4 * k < 3 * I);
      double c = cospi(-1.0 + 2.0 * k / I);
      dayc64[k] = day ? c : 0.0;
      dayc32[k] = day ? (float)c : 0.0f;
    }
  }
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Reference quirk (spectral_transform.py:117-146): the normalisation
// sqrt(((2n+1)(n-m)!) / (2 (n+m)!)) is formed as a correctly rounded float of
// the exact ratio, which for M=106 and m >~ 77 falls into the subnormal range
// (reduced precision) or rounds to 0 (the mode is dropped).  This returns
// sqrt(fl(ratio) / ratio): 1 in the normal range, else the damage factor the
// reference basis carries.  The ratio is accumulated as mantissa * 2^e with
// plain IEEE double operations (relative error < 3e-14, the same on every
// host); the subnormal rounding is then exact up to that error.
static double ref_scale_damage(int m, int n) {
  int e = 0;
  double mant = std::frexp((2.0 * n + 1.0) / 2.0, &e);
  for (int k = n - m + 1; k <= n + m; ++k) {
    int ek = 0;
    mant = std::frexp(mant / (double)k, &ek);
    e += ek;
  }
  // ratio = mant * 2^e, mant in [0.5, 1)
  if (e - 1 >= -1022) return 1.0;               // normal: no damage
  double q = std::ldexp(mant, e + 1074);        // ratio in units of the smallest subnormal
  double k = std::nearbyint(q);
  if (k <= 0.0) return 0.0;
  return std::sqrt(k / q);
}

// Build all static arrays for truncation M into one device allocation.
int geometry_build(GroupGeom& gg, int M, cudaStream_t stream, std::string& err) {
  int J, I;
  if (M == 42) { J = 64; I = 128; }
  else if (M == 63) { J = 96; I = 192; }
  else if (M == 106) { J = 160; I = 320; }
  else { err = "Unsupported value of M=" + std::to_string(M) + ". Only 42, 63, and 106 are supported."; return SWP_ERR_ARG; }
  int N = M, jh = J / 2, L = I / 2;
  std::vector<int> boff(M + 2);
  int acc = 0;
  for (int m = 0; m <= M; ++m) { boff[m] = acc; acc += jh * (N + 1 - m); }
  boff[M + 1] = acc;
  size_t nb = (size_t)acc;
  gg.M = M; gg.J = J; gg.I = I; gg.L = L; gg.nbasis = nb;
  // carve one allocation
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
  size_t o_mu = take(J * 8), o_w = take(J * 8), o_om = take(J * 8), o_area = take(J * 8);
  size_t o_ih64 = take(J * 8), o_cl64 = take(J * 8), o_ih32 = take(J * 4), o_cl32 = take(J * 4);
  size_t o_boff = take((M + 2) * 4);
  size_t o_b64[8], o_b32[8];
  for (int k = 0; k < 8; ++k) o_b64[k] = take(nb * 8);
  for (int k = 0; k < 8; ++k) o_b32[k] = take(nb * 4);
  size_t o_twL64 = take(L * 16), o_twI64 = take((L + 1) * 16), o_twL32 = take(L * 8), o_twI32 = take((L + 1) * 8);
  size_t o_day64 = take(I * 8), o_day32 = take(I * 4), o_err = take(4);
  size_t o_dmg = take((size_t)(M + 1) * (N + 1) * 8);
  cudaError_t e = cudaMalloc(&gg.mem, off);
  if (e != cudaSuccess) { err = std::string("cudaMalloc(geometry): ") + cudaGetErrorString(e); return SWP_ERR_CUDA; }
  gg.bytes = off;
  char* b = (char*)gg.mem;
  gg.mu = (double*)(b + o_mu); gg.w = (double*)(b + o_w); gg.onemu2 = (double*)(b + o_om);
  gg.area = (double*)(b + o_area); gg.boff = (int*)(b + o_boff);
  gg.ihalf64 = (double*)(b + o_ih64); gg.coslat64 = (double*)(b + o_cl64);
  gg.ihalf32 = (float*)(b + o_ih32); gg.coslat32 = (float*)(b + o_cl32);
  for (int k = 0; k < 8; ++k) { gg.b64[k] = (double*)(b + o_b64[k]); gg.b32[k] = (float*)(b + o_b32[k]); }
  gg.twL64 = (double2*)(b + o_twL64); gg.twI64 = (double2*)(b + o_twI64);
  gg.twL32 = (float2*)(b + o_twL32); gg.twI32 = (float2*)(b + o_twI32);
  gg.dayc64 = (double*)(b + o_day64); gg.dayc32 = (float*)(b + o_day32);
  int* derr = (int*)(b + o_err);
  double* ddmg = (double*)(b + o_dmg);
  std::vector<double> dmg((size_t)(M + 1) * (N + 1), 1.0);
  for (int m = 0; m <= M; ++m)
    for (int n = m; n <= N; ++n) dmg[(size_t)m * (N + 1) + n] = ref_scale_damage(m, n);
  cudaMemsetAsync(gg.mem, 0, off, stream);
  cudaMemcpyAsync(gg.boff, boff.data(), (M + 2) * 4, cudaMemcpyHostToDevice, stream);
  cudaMemcpyAsync(ddmg, dmg.data(), dmg.size() * 8, cudaMemcpyHostToDevice, stream);
  k_gauss_nodes<<<(jh + 63) / 64, 64, 0, stream>>>(J, gg.mu, gg.w, derr);
  k_lat_consts<<<(J + 63) / 64, 64, 0, stream>>>(J, I, gg.mu, gg.onemu2, gg.area, gg.ihalf64, gg.coslat64,
                                                 gg.ihalf32, gg.coslat32);
  dim3 gb(M + 1, (jh + 63) / 64);
  k_basis<<<gb, 64, 0, stream>>>(M, J, gg.mu, gg.w, gg.boff, ddmg,
      gg.b64[B_PW_F], gg.b64[B_HW_F], gg.b64[B_P_F], gg.b64[B_H_F],
      gg.b64[B_P_I], gg.b64[B_H_I], gg.b64[B_PW_I], gg.b64[B_HW_I],
      gg.b32[B_PW_F], gg.b32[B_HW_F], gg.b32[B_P_F], gg.b32[B_H_F],
      gg.b32[B_P_I], gg.b32[B_H_I], gg.b32[B_PW_I], gg.b32[B_HW_I]);
  k_twiddles<<<4, 128, 0, stream>>>(I, gg.twL64, gg.twI64, gg.twL32, gg.twI32, gg.dayc64, gg.dayc32);
  int herr = 0;
  cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, stream);
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) { err = std::string("geometry kernels: ") + cudaGetErrorString(e); return SWP_ERR_CUDA; }
  if (herr) { err = "Gauss-Legendre Newton iteration did not converge"; return SWP_ERR_NUMERIC; }
  return SWP_OK;
}

int geometry_dense(const GroupGeom& gg, double* Pd, double* Hd, cudaStream_t stream) {
  k_basis_dense<<<gg.M + 1, 256, 0, stream>>>(gg.M, gg.J, gg.boff, gg.b64[B_P_F], gg.b64[B_H_F], Pd, Hd);
  return cudaGetLastError() == cudaSuccess ? SWP_OK : SWP_ERR_CUDA;
}

}  // namespace swp
