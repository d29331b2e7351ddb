// Per-call coefficient tables of the step kernels (see CoefTables in
// swp_internal.h).  One small launch per library call that runs steps: the
// parameters may change between calls (set_params, gradient sweeps), never
// within one.  The expressions are the ones the reference evaluates:
//   filters.py:95-151          sigma, sigmaPhi (hyperdiffusion), with sigma - 1
//                              and sigmaPhi - 1 formed without cancellation
//   filters.py:154-213         exponential sigma, sigmaPhi (semi-implicit scheme)
//   semi_implicit_tdiff.py     implicit / explicit shares 2 dt si_alpha, 2 dt (1 - si_alpha)
//   model.py:1007-1087         RAW weights alpha w, alpha (1 - w)
//   time_stepping.py:491-534   tstepcoeff, tstepcoeff2, tstepcoeffmn
//   modEuler_tdiff.py:80-261, explicit_tdiff.py:62-226  scalar factors
//   spectral_transform.py:577-594  a / (n(n+1)), omega / sqrt(0.375)
// and, for a tangent-linear call, the derivatives of all of them along the
// members' parameter tangents (a, dt, K6, K6Phi, omega, Phibar).
#include <algorithm>
#include "swp_internal.h"

namespace swp {

template <typename T>
__global__ void k_coefs(const double* __restrict__ par, const double* __restrict__ onemu2, int M, int B, int J,
                        CoefTables<T> C, const double* __restrict__ dpar) {
  const int cnt = M + 1;
  const int n_nco = B * cnt, n_jco = B * J;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_nco + n_jco + B; t += gridDim.x * blockDim.x) {
    if (t < n_nco) {
      const int b = t / cnt, n = t % cnt;
      const double a = par[P_A * B + b], dt = par[P_DT * B + b];
      const double K6 = par[P_K6 * B + b], K6P = par[P_K6PHI * B + b];
      const double nd = (double)n;
      const double ncoeff = ((nd * nd * nd) / (a * a * a)) * (((nd + 1) * (nd + 1) * (nd + 1)) / (a * a * a));
      const double a6 = a * a * a * a * a * a;
      const double x = 2.0 * dt * K6 * (ncoeff - 8.0 / a6), xp = 2.0 * dt * K6P * ncoeff;
      const size_t o = (size_t)b * cnt + n, qs = (size_t)B * cnt;
      C.nco[NC_SIG * qs + o] = (T)(1.0 / (1.0 + x));
      C.nco[NC_SIGP * qs + o] = (T)(1.0 / (1.0 + xp));
      C.nco[NC_SIGM1 * qs + o] = (T)(-x / (1.0 + x));
      C.nco[NC_SIGPM1 * qs + o] = (T)(-xp / (1.0 + xp));
      C.nco[NC_TC * qs + o] = (T)((n == 0) ? 0.0 : a / ((double)n * (n + 1)));
      C.nco[NC_SIGX * qs + o] = (T)exp(-(2.0 * dt * K6) * fmax(ncoeff - 8.0 / a6, 0.0));
      C.nco[NC_SIGPX * qs + o] = (T)exp(-(2.0 * dt * K6P) * ncoeff);
      // tangents: sigma = 1/(1+x) -> -sigma^2 dx, with x = 2 dt K6 r, r ~ a^-6
      double dsig = 0.0, dsigp = 0.0, dtc = 0.0;
      if (dpar) {
        const double da = dpar[T_A * B + b], ddt = dpar[T_DT * B + b];
        const double dK6 = dpar[T_K6 * B + b], dK6P = dpar[T_K6PHI * B + b];
        const double r = ncoeff - 8.0 / a6, s1 = 1.0 / (1.0 + x), s2 = 1.0 / (1.0 + xp);
        const double dx = 2.0 * ddt * K6 * r + 2.0 * dt * dK6 * r - 6.0 * (da / a) * x;
        const double dxp = 2.0 * ddt * K6P * ncoeff + 2.0 * dt * dK6P * ncoeff - 6.0 * (da / a) * xp;
        dsig = -s1 * s1 * dx;
        dsigp = -s2 * s2 * dxp;
        dtc = (n == 0) ? 0.0 : da / ((double)n * (n + 1));
      }
      // exponential sigmas: exp(-2 dt K6 max(r, 0)), exp(-2 dt K6Phi ncoeff)
      double dsigx = 0.0, dsigpx = 0.0;
      if (dpar) {
        const double da = dpar[T_A * B + b], ddt = dpar[T_DT * B + b];
        const double dK6 = dpar[T_K6 * B + b], dK6P = dpar[T_K6PHI * B + b];
        const double r = fmax(ncoeff - 8.0 / a6, 0.0);
        const double dr = r > 0.0 ? -6.0 * (da / a) * r : 0.0, dnc = -6.0 * (da / a) * ncoeff;
        dsigx = -exp(-(2.0 * dt * K6) * r) * (2.0 * ddt * K6 * r + 2.0 * dt * dK6 * r + 2.0 * dt * K6 * dr);
        dsigpx = -exp(-(2.0 * dt * K6P) * ncoeff) * (2.0 * ddt * K6P * ncoeff + 2.0 * dt * dK6P * ncoeff +
                                                     2.0 * dt * K6P * dnc);
      }
      C.nco[NC_DSIG * qs + o] = (T)dsig;
      C.nco[NC_DSIGP * qs + o] = (T)dsigp;
      C.nco[NC_DTC * qs + o] = (T)dtc;
      C.nco[NC_DSIGX * qs + o] = (T)dsigx;
      C.nco[NC_DSIGPX * qs + o] = (T)dsigpx;
    } else if (t < n_nco + n_jco) {
      const int u = t - n_nco, b = u / J, j = u % J;
      const double a = par[P_A * B + b], dt = par[P_DT * B + b];
      const double tsc = (2.0 * dt) / (a * onemu2[j]);
      C.jco[u] = (T)tsc;
      C.djco[u] = (T)(dpar ? (2.0 * dpar[T_DT * B + b]) / (a * onemu2[j]) - tsc * dpar[T_A * B + b] / a : 0.0);
    } else {
      const int b = t - n_nco - n_jco;
      const double a = par[P_A * B + b], dt = par[P_DT * B + b], Pb = par[P_PHIBAR * B + b];
      const double td = par[P_TAUDRAG * B + b], om = par[P_OMEGA * B + b];
      T* mc = C.mco;
      mc[MC_DT * B + b] = (T)dt;
      mc[MC_T2 * B + b] = (T)((2.0 * dt / (a * a)) / 4.0);
      mc[MC_IA2 * B + b] = (T)(1.0 / (a * a));
      mc[MC_HPB * B + b] = (T)(Pb * 0.5);
      mc[MC_DTPB * B + b] = (T)(dt * Pb);
      mc[MC_PBA2 * B + b] = (T)(Pb / (a * a));
      mc[MC_PFD * B + b] = (T)((dt / 2.0) / (a * a));
      mc[MC_2DTPB * B + b] = (T)(2.0 * dt * Pb);
      mc[MC_2DT * B + b] = (T)(2.0 * dt);
      mc[MC_ITD * B + b] = (T)(1.0 / td);
      mc[MC_OM * B + b] = (T)(om / sqrt(0.375));
      const double al = par[P_ALPHA * B + b], sa = par[P_SIALPHA * B + b], wa = par[P_WALPHA * B + b];
      mc[MC_ALPHA * B + b] = (T)al;
      mc[MC_SIXI * B + b] = (T)(2.0 * dt * sa);
      mc[MC_SIEX * B + b] = (T)(2.0 * dt * (1.0 - sa));
      mc[MC_SIITD * B + b] = (T)(td == -1.0 ? 0.0 : 1.0 / td);
      mc[MC_SIITR * B + b] = (T)(1.0 / par[P_TAURAD * B + b]);
      mc[MC_RAWM * B + b] = (T)(al * wa);
      mc[MC_RAWN * B + b] = (T)(al * (1.0 - wa));
      mc[MC_PB * B + b] = (T)Pb;
      double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (dpar) {
        const double da = dpar[T_A * B + b], ddt = dpar[T_DT * B + b], dPb = dpar[T_PHIBAR * B + b];
        const double dom = dpar[T_OMEGA * B + b], a3 = a * a * a;
        v[0] = (2.0 * ddt / (a * a) - 4.0 * dt * da / a3) / 4.0;  // (2 dt / a^2) / 4
        v[1] = -2.0 * da / a3;                                    // 1 / a^2
        v[2] = dPb * 0.5;                                          // Phibar / 2
        v[3] = ddt * Pb + dt * dPb;                                // dt Phibar
        v[4] = dPb / (a * a) - 2.0 * Pb * da / a3;                 // Phibar / a^2
        v[5] = (ddt / 2.0) / (a * a) - dt * da / a3;               // (dt / 2) / a^2
        v[6] = ddt;                                                // dt
        v[7] = dom / sqrt(0.375);                                  // omega / sqrt(0.375)
      }
      const int dr[8] = {MC_DT2, MC_DIA2, MC_DHPB, MC_DDTPB, MC_DPBA2, MC_DPFD, MC_DDT, MC_DOM};
      for (int q = 0; q < 8; ++q) mc[dr[q] * B + b] = (T)v[q];
      // semi-implicit: xi = 2 dt sa, ex = 2 dt (1 - sa), 1/taudrag (0 for -1), 1/taurad
      double w[4] = {0, 0, 0, 0};
      if (dpar) {
        const double ddt = dpar[T_DT * B + b], dsa = dpar[T_SIALPHA * B + b];
        const double itd = td == -1.0 ? 0.0 : 1.0 / td, itr = 1.0 / par[P_TAURAD * B + b];
        w[0] = 2.0 * ddt * sa + 2.0 * dt * dsa;
        w[1] = 2.0 * ddt * (1.0 - sa) - 2.0 * dt * dsa;
        w[2] = -itd * itd * dpar[T_TAUDRAG * B + b];
        w[3] = -itr * itr * dpar[T_TAURAD * B + b];
      }
      mc[MC_DSIXI * B + b] = (T)w[0];
      mc[MC_DSIEX * B + b] = (T)w[1];
      mc[MC_DSIITD * B + b] = (T)w[2];
      mc[MC_DSIITR * B + b] = (T)w[3];
      mc[MC_DITD * B + b] = (T)(dpar ? -dpar[T_TAUDRAG * B + b] / (td * td) : 0.0);
      // the filter weights: alpha (classic), alpha wa and alpha (1 - wa) (RAW)
      const double dal = dpar ? dpar[T_ALPHA * B + b] : 0.0, dwa = dpar ? dpar[T_WALPHA * B + b] : 0.0;
      mc[MC_DALPHA * B + b] = (T)dal;
      mc[MC_DRAWM * B + b] = (T)(dal * wa + al * dwa);
      mc[MC_DRAWN * B + b] = (T)(dal * (1.0 - wa) - al * dwa);
    }
  }
}

template <typename T>
cudaError_t launch_coefs(const double* par, const double* onemu2, int M, int B, int J, const CoefTables<T>& C,
                         cudaStream_t s, const double* dpar) {
  const int total = B * (M + 1) + B * J + B;
  const int nb = std::min((total + 255) / 256, 1216);
  k_coefs<T><<<nb, 256, 0, s>>>(par, onemu2, M, B, J, C, dpar);
  return cudaGetLastError();
}
template cudaError_t launch_coefs<double>(const double*, const double*, int, int, int, const CoefTables<double>&,
                                          cudaStream_t, const double*);
template cudaError_t launch_coefs<float>(const double*, const double*, int, int, int, const CoefTables<float>&,
                                         cudaStream_t, const double*);

}  // namespace swp
