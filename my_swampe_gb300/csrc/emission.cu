// Emission stage of the retrieval, batched over ensemble members, in FP64 like
// the reference (whose emission / light-curve stage stays float64 even when the
// dynamics run in float32).  It maps a member's terminal Phi to the
// spherical-harmonic coefficients of its emission map and to a phase curve:
//
//   phi_to_temperature            retrieval/scripts/pipeline.py:696-714
//   temperature_to_intensity      pipeline.py:716-754 (bolometric T^4, or the
//                                 relative Planck intensity, optionally band-averaged)
//   intensity_map_to_y_dense      pipeline.py:821-846 (weighted ridge least-squares
//                                 projection onto the Ylm basis, normalised by y0)
//   the planet's light curve      pipeline.py:983-994: linear in the map
//                                 coefficients, amplitude planet_fpfs
//   the simplified phase curve    unit_tests/test_parity_reference_regression.py:67-82
//
// The Ylm design matrix and the light-curve design matrix come from a
// third-party model (jaxoplanet 0.1.0, starry Surface.intensity and
// light_curve) that the caller evaluates once; the projector built from the
// former is an input here, as in the reference, which builds it once per
// pipeline (pipeline.py:808-819).
//
// Every kernel's reductions run in a fixed order, so results are reproducible
// run to run.  Non-finite inputs give all-NaN outputs per member, as the
// reference's lax.cond guards do.
#include <cmath>
#include "swp_internal.h"

namespace swp {
namespace {

constexpr int EM_THREADS = 256;

// FP64 block sum of one value per thread (fixed order: warp shuffles, then
// warp 0 over the 8 warp slots); every thread gets the total.
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();  // red may still be read from the previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double s = lane < EM_THREADS / 32 ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[EM_THREADS / 32] = s;
  }
  __syncthreads();
  return red[EM_THREADS / 32];
}
__device__ bool block_all(bool v) { return __syncthreads_and(v ? 1 : 0) != 0; }

struct EmCfg {
  int temp_mode, model, nbands, input;  // input: 0 = Phi, 1 = T, 2 = intensity
  double R_d, T_ref, phi_to_T_scale, Tmin, x_clip;
  double wl[SWP_EMISSION_MAX_BANDS], bw[SWP_EMISSION_MAX_BANDS];
};

__device__ __forceinline__ double temperature(const EmCfg& c, double phi, double Phibar) {
  const double T = c.temp_mode == 0 ? (Phibar + phi) / c.R_d : c.T_ref + phi / c.phi_to_T_scale;
  return fmax(T, c.Tmin);
}
// relative Planck intensity 1 / (expm1(x) + tiny), x = h c / (lambda kB T)
// clipped to [0, x_clip] (pipeline.py:716-735)
__device__ __forceinline__ double planck_rel(double T, double lam, double x_clip) {
  const double h = 6.62607015e-34, c = 299792458.0, kB = 1.380649e-23;
  double x = (h * c) / (lam * kB * T);
  x = fmin(fmax(x, 0.0), x_clip);
  return 1.0 / (expm1(x) + 1.0e-30);
}
__device__ __forceinline__ double intensity(const EmCfg& c, double T) {
  if (c.model == 0) {
    const double t2 = T * T;
    return t2 * t2;
  }
  double out = 0.0;
  for (int k = 0; k < c.nbands; ++k) out += c.bw[k] * planck_rel(T, c.wl[k], c.x_clip);
  return out;
}

// One CTA per member.  stage 0 writes T, 1 the intensity map, 2 the weighted
// relative intensity w_sqrt I / I_mean that the projector multiplies (and
// ok[b] = the map's guards passed).  The passes follow the reference's guards:
// a non-finite Phi makes T all NaN; a non-finite T makes the Planck intensity
// all NaN; the relative map needs a finite, nonzero weighted mean.
__global__ void __launch_bounds__(EM_THREADS) k_emission_map(const double* __restrict__ in,
                                                             const double* __restrict__ Phibar, int J, int I,
                                                             const double* __restrict__ w_lat, EmCfg c, int stage,
                                                             double* __restrict__ out, int* __restrict__ ok) {
  __shared__ double red[EM_THREADS / 32 + 1];
  const int b = blockIdx.x;
  const size_t npix = (size_t)J * I;
  const double* x = in + (size_t)b * npix;
  double* y = out + (size_t)b * npix;
  const double pb = Phibar ? Phibar[b] : 0.0;
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  // pass 1: all of the input finite (Phi -> T guard; a T or intensity input
  // enters the guard of its own stage below)
  bool fin = true;
  for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) fin &= isfinite(x[p]) != 0;
  const bool in_ok = block_all(fin);
  auto T_at = [&](size_t p) { return c.input == 0 ? (in_ok ? temperature(c, x[p], pb) : qnan) : x[p]; };
  if (stage == 0) {
    for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) y[p] = T_at(p);
    return;
  }
  // pass 2: the Planck guard needs every T finite
  bool t_ok = true;
  if (c.input <= 1 && c.model == 1) {
    bool ft = true;
    for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) ft &= isfinite(T_at(p)) != 0;
    t_ok = block_all(ft);
  }
  auto I_at = [&](size_t p) {
    if (c.input == 2) return x[p];
    const double T = T_at(p);
    return (c.model == 1 && !t_ok) ? qnan : intensity(c, T);
  };
  if (stage == 1) {
    for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) y[p] = I_at(p);
    return;
  }
  // pass 3: the weighted mean over the finite pixels (pipeline.py:821-837)
  double sw = 0.0, swi = 0.0;
  bool fi = true;
  for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) {
    const double v = I_at(p);
    const double w = w_lat[p / I];
    const bool f = isfinite(v) != 0;
    fi &= f;
    if (f) {
      sw += w;
      swi += w * v;
    }
    y[p] = v;  // kept for pass 4
  }
  const bool all_fin = block_all(fi);
  const double w_sum = block_sum(sw, red);
  const double wi_sum = block_sum(swi, red);
  const double mean = w_sum > 0.0 ? wi_sum / w_sum : qnan;
  const bool mean_ok = isfinite(mean) && fabs(mean) > 1.0e-30;
  // pass 4: rhs = sqrt(w) * I_rel, I_rel = I / mean (NaN where I is not finite or the mean fails)
  for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) {
    const double v = y[p];
    const double safe = isfinite(v) ? v : 0.0;
    y[p] = sqrt(w_lat[p / I]) * (mean_ok ? safe / mean : qnan);
  }
  if (threadIdx.x == 0 && ok) ok[b] = (all_fin && mean_ok) ? 1 : 0;
}

// Y[b][c] = sum_p P[c][p] rhs[b][p]: one CTA per (member, 32 coefficients),
// a warp per 4 coefficients, lanes over pixels, fixed-order warp sums.
__global__ void __launch_bounds__(EM_THREADS) k_emission_project(const double* __restrict__ rhs, int npix,
                                                                 const double* __restrict__ P, int ncoef,
                                                                 double* __restrict__ yraw) {
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = blockIdx.x * 32 + warp * 4;
  const double* r = rhs + (size_t)b * npix;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int p = lane; p < npix; p += 32) {
    const double v = r[p];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (c0 + q < ncoef) acc[q] = fma(P[(size_t)(c0 + q) * npix + p], v, acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    double s = acc[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0 && c0 + q < ncoef) yraw[(size_t)b * ncoef + c0 + q] = s;
  }
}

// y / y0 with the reference's guards (pipeline.py:838-846): one warp per member.
__global__ void k_emission_normalise(const int* __restrict__ ok, int B, int ncoef, double* __restrict__ y) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (b >= B) return;
  double* v = y + (size_t)b * ncoef;
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  const double y0 = v[0];
  const bool y0_ok = isfinite(y0) && fabs(y0) > 1.0e-30;
  bool fin = true;
  for (int c = lane; c < ncoef; c += 32) fin &= isfinite(y0_ok ? v[c] / y0 : qnan) != 0;
  fin = __all_sync(0xffffffffu, fin);
  const bool good = (ok ? ok[b] != 0 : true) && y0_ok && fin;
  __syncwarp();
  for (int c = lane; c < ncoef; c += 32) v[c] = good ? v[c] / y0 : qnan;
}

// lc[b][t] = amplitude[b] * sum_c A[t][c] y[b][c]
__global__ void k_phase_curve_linear(const double* __restrict__ y, const double* __restrict__ A,
                                     const double* __restrict__ amp, int B, int ncoef, int ntimes,
                                     double* __restrict__ lc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * ntimes) return;
  const int b = i / ntimes, t = i % ntimes;
  const double* yv = y + (size_t)b * ncoef;
  const double* a = A + (size_t)t * ncoef;
  double s = 0.0;
  for (int c = 0; c < ncoef; ++c) s = fma(a[c], yv[c], s);
  lc[i] = (amp ? amp[b] : 1.0) * s;
}

// flux[b][k] = sum_{j,i} Phi max(cos(lambda_i - phase_k), 0) sqrt(1 - mu_j^2),
// then divided by mean_k |flux| when that is positive: one CTA per member.
__global__ void __launch_bounds__(EM_THREADS) k_phase_curve_simple(const double* __restrict__ phi, int J, int I,
                                                                   const double* __restrict__ mus,
                                                                   const double* __restrict__ phases, int nph,
                                                                   double* __restrict__ flux) {
  __shared__ double red[EM_THREADS / 32 + 1];
  const int b = blockIdx.x;
  const size_t npix = (size_t)J * I;
  const double* x = phi + (size_t)b * npix;
  double* f = flux + (size_t)b * nph;
  const double pi = 3.141592653589793, step = (pi - (-pi)) / I;  // numpy linspace(-pi, pi, I, endpoint=False)
  double asum = 0.0;
  for (int k = 0; k < nph; ++k) {
    const double ph = phases[k];
    double s = 0.0;
    for (size_t p = threadIdx.x; p < npix; p += EM_THREADS) {
      const int j = (int)(p / I), i = (int)(p % I);
      const double mu = mus[j];
      const double aw = sqrt(fmax(1.0 - mu * mu, 0.0));
      const double vis = fmax(cos((-pi + i * step) - ph), 0.0);
      s += x[p] * vis * aw;
    }
    const double tot = block_sum(s, red);
    if (threadIdx.x == 0) f[k] = tot;
    asum += fabs(tot);
  }
  const double norm = asum / nph;
  __syncthreads();
  if (norm > 0.0)
    for (int k = threadIdx.x; k < nph; k += EM_THREADS) f[k] = f[k] / norm;
}

int em_check(cudaError_t e) { return e == cudaSuccess ? SWP_OK : SWP_ERR_CUDA; }

}  // namespace
}  // namespace swp

using namespace swp;

extern "C" int swp_emission_map(const double* in, const double* Phibar, int B, int J, int I, const double* w_lat,
                                const swp_emission_cfg* cfg, int input, int stage, double* out, int* ok,
                                void* stream) {
  if (!in || !cfg || !out || B < 1 || J < 1 || I < 1 || stage < 0 || stage > 2 || input < 0 || input > 2)
    return SWP_ERR_ARG;
  if (input > stage) return SWP_ERR_ARG;                 // the stage is computed from an earlier one
  if (input == 0 && !Phibar && cfg->temp_mode == 0) return SWP_ERR_ARG;
  if (stage == 2 && !w_lat) return SWP_ERR_ARG;
  if (cfg->temp_mode < 0 || cfg->temp_mode > 1 || cfg->model < 0 || cfg->model > 1) return SWP_ERR_ARG;
  if (cfg->model == 1 && (cfg->nbands < 1 || cfg->nbands > SWP_EMISSION_MAX_BANDS)) return SWP_ERR_ARG;
  EmCfg c;
  c.temp_mode = cfg->temp_mode;
  c.model = cfg->model;
  c.nbands = cfg->model == 1 ? cfg->nbands : 0;
  c.input = input;
  c.R_d = cfg->R_d;
  c.T_ref = cfg->T_ref;
  c.phi_to_T_scale = cfg->phi_to_T_scale;
  c.Tmin = cfg->Tmin;
  c.x_clip = cfg->x_clip;
  for (int k = 0; k < SWP_EMISSION_MAX_BANDS; ++k) {
    c.wl[k] = k < c.nbands ? cfg->wavelengths[k] : 1.0;
    c.bw[k] = k < c.nbands ? cfg->band_weights[k] : 0.0;
  }
  k_emission_map<<<B, EM_THREADS, 0, (cudaStream_t)stream>>>(in, Phibar, J, I, w_lat, c, stage, out, ok);
  return em_check(cudaGetLastError());
}

extern "C" int swp_emission_project(const double* rhs, const int* ok, int B, int npix, const double* projector,
                                    int ncoef, double* y, void* stream) {
  if (!rhs || !projector || !y || B < 1 || npix < 1 || ncoef < 1 || B > 65535) return SWP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((ncoef + 31) / 32, B);
  k_emission_project<<<grid, EM_THREADS, 0, s>>>(rhs, npix, projector, ncoef, y);
  if (cudaError_t e = cudaGetLastError()) return em_check(e);
  k_emission_normalise<<<(B + 7) / 8, 256, 0, s>>>(ok, B, ncoef, y);
  return em_check(cudaGetLastError());
}

extern "C" int swp_phase_curve_linear(const double* y, const double* design, const double* amplitude, int B,
                                      int ncoef, int ntimes, double* lc, void* stream) {
  if (!y || !design || !lc || B < 1 || ncoef < 1 || ntimes < 1) return SWP_ERR_ARG;
  const long long n = (long long)B * ntimes;
  if (n > (1ll << 31) - 1) return SWP_ERR_ARG;
  k_phase_curve_linear<<<(int)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(y, design, amplitude, B, ncoef,
                                                                                 ntimes, lc);
  return em_check(cudaGetLastError());
}

extern "C" int swp_phase_curve_simple(const double* phi, int B, int J, int I, const double* mus,
                                      const double* phases, int nphase, double* flux, void* stream) {
  if (!phi || !mus || !phases || !flux || B < 1 || J < 1 || I < 1 || nphase < 1) return SWP_ERR_ARG;
  k_phase_curve_simple<<<B, EM_THREADS, 0, (cudaStream_t)stream>>>(phi, J, I, mus, phases, nphase, flux);
  return em_check(cudaGetLastError());
}
