// Pieces shared by the SIMT and tensor-core Legendre kernels of a step:
// the combined-input slots and their evaluation at one (m, member, latitude).
#pragma once
#include "swp_internal.h"

namespace swp {

// combined-input slots of the forward contraction.  The FP32 path carries three
// more P slots (the current eta, delta, Phi on their own) for the incremental
// form of the step; the FP64 path keeps the reference's projection form.
enum SlotP { SP_PHI1 = 0, SP_PHI2, SP_D1, SP_D2, SP_E1, SP_IPHI, SP_ID, SP_IE };  // on Pw
enum SlotH { SH_PHI1 = 0, SH_D1, SH_D2, SH_E1, NSH };                            // on Hw
template <typename T> struct SlotCount { static constexpr int NP = 5; static constexpr bool INCR = false; };
template <> struct SlotCount<float> { static constexpr int NP = 8; static constexpr bool INCR = true; };
constexpr int NSP = 5;
template <typename T>
__device__ __forceinline__ const SpecGroup<T>& pick_group(const SpecLaunch<T>& L, int& idx) {
  int gi = 0;
  while (gi + 1 < L.ng && (int)blockIdx.x >= L.prefix[gi + 1]) ++gi;
  idx = blockIdx.x - L.prefix[gi];
  return L.grp[gi];
}

// i*m*z
template <typename T2, typename T>
__device__ __forceinline__ T2 imul(T m, T2 z) { T2 r; r.x = -m * z.y; r.y = m * z.x; return r; }

// Per-(member, n) spectral coefficients of a CTA's tile from the call's tables
// into shared memory; without hyperdiffusion sigma = 1, sigma - 1 = 0.  `expo`
// selects the exponential sigmas of the semi-implicit scheme.
template <typename T>
__device__ __forceinline__ void load_spec_coefs(const SpecGroup<T>& G, bool diff, int m, int b0, int mt, int MT,
                                                int cnt, int cntmax, T* sig, T* sigP, T* sigm1, T* sigPm1, T* tcmn,
                                                bool expo = false) {
  const size_t qs = (size_t)G.B * cntmax;
  const int rs = expo ? NC_SIGX : NC_SIG, rp = expo ? NC_SIGPX : NC_SIGP;
  for (int t = threadIdx.x; t < MT * cnt; t += blockDim.x) {
    const int bt = t / cnt, k = t % cnt, n = m + k;
    T s = (T)1, sp = (T)1, sm1 = (T)0, spm1 = (T)0, tc = (T)0;
    if (bt < mt) {
      const size_t o = (size_t)(b0 + bt) * cntmax + n;
      if (diff) {
        s = G.nco[rs * qs + o];
        sp = G.nco[rp * qs + o];
        sm1 = G.nco[NC_SIGM1 * qs + o];
        spm1 = G.nco[NC_SIGPM1 * qs + o];
      }
      tc = G.nco[NC_TC * qs + o];
    }
    sig[bt * cntmax + k] = s;
    sigP[bt * cntmax + k] = sp;
    sigm1[bt * cntmax + k] = sm1;
    sigPm1[bt * cntmax + k] = spm1;
    tcmn[bt * cntmax + k] = tc;
  }
}

// The per-point step factors of the modified-Euler combination: tstepcoeff at
// (member, latitude) and the member's 2dt/a^2/4, 1/a^2, Phibar/2, dt Phibar,
// Phibar/a^2, dt/(2a^2) and dt.  The tensor-core step loads them while its
// input copies are in flight; the other callers read them in place.
template <typename T>
struct StepCoefs {
  T tsc, t2, ia2, hpb, dtpb, pba2, pfd, dt;
};
template <typename T>
__device__ __forceinline__ StepCoefs<T> load_step_coefs(const SpecGroup<T>& G, int b, int j) {
  const T* mc = G.mco;
  const int B = G.B;
  StepCoefs<T> k;
  k.tsc = G.jco[(size_t)b * G.g.J + j];
  k.t2 = mc[MC_T2 * B + b];
  k.ia2 = mc[MC_IA2 * B + b];
  k.hpb = mc[MC_HPB * B + b];
  k.dtpb = mc[MC_DTPB * B + b];
  k.pba2 = mc[MC_PBA2 * B + b];
  k.pfd = mc[MC_PFD * B + b];
  k.dt = mc[MC_DT * B + b];
  return k;
}

// The combined inputs of the forward contraction at (m, member b, latitude j):
// every reference tendency term that is a Legendre transform of a pointwise
// product of Fourier inputs (modEuler_tdiff.py:72-110, 162-201, 253-261;
// explicit_tdiff.py:62-78, 134-155, 207-226), grouped by the basis (Pw or Hw)
// and by the output factor (1 or n(n+1)) they are applied with.  mode 2 is the
// plain transform of eta, delta used to diagnose winds (model.py:644-666).
// `ld(f)` returns Fourier field f at the point (from global memory or a staged copy).
// `kc`, if given, holds the point's step factors (modified Euler), loaded ahead.
template <typename T, typename LD>
__device__ __forceinline__ void step_combos_ld(const SpecGroup<T>& G, const StepCfg& cfg, int mode, bool incr, int m,
                                               int b, int j, LD ld, typename cplx<T>::type* c,
                                               const StepCoefs<T>* kc = nullptr) {
  typedef typename cplx<T>::type T2;
  constexpr int NSPX = SlotCount<T>::NP;
  constexpr int NSLOT = NSPX + NSH;
  const Geom<T>& g = G.g;
  const T* mc = G.mco;
  const int B = G.B;
  const T xm = (T)m;
  const T tsc = kc ? kc->tsc : G.jco[(size_t)b * g.J + j];  // tstepcoeff
  T2 z = mk<T2>(0, 0);
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) c[q] = z;
  if (mode == 2) {  // diagnose winds: plain forward transforms of eta, delta
    c[SP_E1] = ld(F_ETA);
    c[SP_D1] = ld(F_DELTA);
  } else if (cfg.scheme == 0) {
    T2 eta = ld(F_ETA), del = ld(F_DELTA), phi = ld(F_PHI);
    T2 A = ld(F_A), Bm = ld(F_B), C = ld(F_C), D = ld(F_D);
    T2 E = ld(F_E), PF = ld(F_PHIF), Fm = ld(F_F), Gm = ld(F_G);
    const StepCoefs<T> k = kc ? *kc : load_step_coefs<T>(G, b, j);
    T t1 = tsc * (T)0.25, t2 = k.t2;
    T ia2 = k.ia2;
    T hPb = k.hpb;
    T2 Bf = cadd(Bm, Fm), Af = csub(A, Gm);
    T2 Beff = cfg.forcflag ? Bf : Bm, Aeff = cfg.forcflag ? Af : A;
    // Phi (modEuler_tdiff.py:80-110); incremental form: curr goes to its own slot
    T2 p1 = incr ? cscale(imul(xm, C), -t1) : csub(phi, cscale(imul(xm, C), t1));
    p1 = csub(p1, cscale(del, k.dtpb));
    p1 = csub(p1, cscale(imul(xm, Beff), hPb * t1));
    if (cfg.forcflag) p1 = cadd(p1, cscale(PF, k.dt));
    c[SP_PHI1] = p1;
    c[NSPX + SH_PHI1] = csub(cscale(D, t1), cscale(Aeff, hPb * t1));
    c[SP_PHI2] = cscale(cadd(cscale(E, t2), cscale(phi, ia2)), -hPb);
    // delta (modEuler_tdiff.py:162-201)
    c[SP_D1] = incr ? cscale(imul(xm, Bf), t1) : cadd(del, cscale(imul(xm, Bf), t1));
    c[NSPX + SH_D1] = cscale(Af, t1);
    T2 d2 = cadd(cscale(phi, t2), cscale(E, t2));
    d2 = cadd(d2, cscale(imul(xm, C), t1 * (T)0.5 * ia2));
    d2 = csub(d2, cscale(del, k.pba2));
    if (cfg.forcflag) d2 = cadd(d2, cscale(PF, k.pfd));
    c[SP_D2] = d2;
    c[NSPX + SH_D2] = cscale(D, t1 * (T)0.5 * ia2);
    // eta (modEuler_tdiff.py:253-261)
    T te = cfg.forcflag ? tsc : tsc * (T)0.5;
    c[SP_E1] = incr ? cscale(imul(xm, Aeff), -te) : csub(eta, cscale(imul(xm, Aeff), te));
    c[NSPX + SH_E1] = cscale(Beff, te);
    if (incr) { c[SP_IPHI] = phi; c[SP_ID] = del; c[SP_IE] = eta; }
  } else if (cfg.scheme == 2) {
    // semi-implicit leapfrog (semi_implicit_tdiff.py si_timestep): explicit
    // parts of eta*, delta*, Phi* on the n-1 base (the filtered lineage);
    // SP_D2 carries the terms applied with n(n+1)/a^2, the rest factor 1.
    // The per-degree implicit solve is the spectral kernel's epilogue.
    T2 eta0 = ld(F_ETA_MID), del0 = ld(F_DELTA_MID), phi0 = ld(F_PHI_MID);
    T2 A = ld(F_A), Bm = ld(F_B), C = ld(F_C), D = ld(F_D), E = ld(F_E);
    const T ex = mc[MC_SIEX * B + b];
    const T itd = cfg.si_relax ? mc[MC_SIITD * B + b] : (T)0;
    const T itr = cfg.si_relax ? mc[MC_SIITR * B + b] : (T)0;
    const T gd = ex * itd, gr = ex * itr, tdt = mc[MC_2DT * B + b];
    T2 Aeff = A, Beff = Bm, PFx = mk<T2>(0, 0);
    if (cfg.forcflag) {
      T2 Fx, Gx;
      if (cfg.si_relax) {
        // lagged remainder Fm + Um / taudrag of the previous step; on the first
        // step the state's own (model.py:737-739)
        if (cfg.si_lag_init) {
          Fx = cadd(ld(F_F), cscale(ld(F_U), itd));
          Gx = cadd(ld(F_G), cscale(ld(F_V), itd));
        } else {
          Fx = ld(F_RU_LAG);
          Gx = ld(F_RV_LAG);
        }
        PFx = cadd(ld(F_PHIF), cscale(ld(F_PHI), itr));
      } else {
        Fx = ld(F_F);
        Gx = ld(F_G);
        PFx = ld(F_PHIF);
      }
      Aeff = csub(A, Gx);
      Beff = cadd(Bm, Fx);
    }
    T2 e1 = csub(cscale(eta0, (T)1 - gd), cscale(imul(xm, Aeff), tsc));
    T2 d1 = cadd(cscale(del0, (T)1 - gd), cscale(imul(xm, Beff), tsc));
    T2 p1 = csub(cscale(phi0, (T)1 - gr), cscale(imul(xm, C), tsc));
    p1 = csub(p1, cscale(del0, ex * mc[MC_PB * B + b]));
    if (cfg.forcflag) p1 = cadd(p1, cscale(PFx, tdt));
    c[SP_E1] = e1;
    c[SP_D1] = d1;
    c[SP_PHI1] = p1;
    c[SP_D2] = cscale(cadd(cscale(E, tdt), cscale(phi0, ex)), mc[MC_IA2 * B + b]);
    c[NSPX + SH_E1] = cscale(Beff, tsc);
    c[NSPX + SH_D1] = cscale(Aeff, tsc);
    c[NSPX + SH_PHI1] = cscale(D, tsc);
  } else {
    T2 eta0 = ld(F_ETA_PREV), del0 = ld(F_DELTA_PREV), phi0 = ld(F_PHI_PREV);
    T2 del1 = ld(F_DELTA);
    T2 A = ld(F_A), Bm = ld(F_B), C = ld(F_C), D = ld(F_D);
    T2 PF = ld(F_PHIF), Fm = ld(F_F), Gm = ld(F_G);
    T2 U = ld(F_U), V = ld(F_V);
    T t = tsc;
    T itd = mc[MC_ITD * B + b];
    // Phi (explicit_tdiff.py:62-78)
    T2 p1 = csub(phi0, cscale(imul(xm, C), t));
    p1 = csub(p1, cscale(del1, mc[MC_2DTPB * B + b]));
    if (cfg.forcflag) p1 = cadd(p1, cscale(PF, mc[MC_2DT * B + b]));
    c[SP_PHI1] = p1;
    c[NSPX + SH_PHI1] = cscale(D, t);
    // delta (explicit_tdiff.py:134-155)
    T2 d1 = del0, dh = mk<T2>(0, 0);
    if (cfg.forcflag) {
      d1 = csub(d1, cscale(imul(xm, U), t * itd));
      d1 = cadd(d1, cscale(imul(xm, Fm), t));
      dh = csub(cscale(V, t * itd), cscale(Gm, t));
    }
    c[SP_D1] = d1;
    c[NSPX + SH_D1] = dh;
    // eta (explicit_tdiff.py:207-226)
    T2 e1 = csub(eta0, cscale(imul(xm, A), t));
    T2 eh = cscale(Bm, t);
    if (cfg.forcflag) {
      e1 = csub(e1, cscale(imul(xm, V), t * itd));
      e1 = cadd(e1, cscale(imul(xm, Gm), t));
      eh = cadd(eh, cscale(U, t * itd));
      eh = cadd(eh, cscale(Fm, t));
    }
    c[SP_E1] = e1;
    c[NSPX + SH_E1] = eh;
  }
}

// Tangent-linear step (modified Euler): the combined inputs are linear in the
// state, with coefficients that depend on the parameters (modEuler_tdiff.py:
// 72-110, 162-201, 253-261): their tangent is step_combos on the tangent state
// plus the tangents of the coefficients (the call's tables: tstepcoeff and the
// scalar factors, along the members' tangents of a, dt and Phibar) times the
// primal state before the step, `four_p`.
template <typename T>
__device__ __forceinline__ void tangent_coef_terms_si(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                      size_t FS, typename cplx<T>::type* c);
template <typename T>
__device__ __forceinline__ void tangent_coef_terms_ex(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                      size_t FS, typename cplx<T>::type* c);

template <typename T>
__device__ __forceinline__ void tangent_coef_terms(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                   size_t FS, typename cplx<T>::type* c) {
  if (cfg.scheme == 2) {
    tangent_coef_terms_si<T>(G, cfg, m, b, j, FS, c);
    return;
  }
  if (cfg.scheme == 1) {
    tangent_coef_terms_ex<T>(G, cfg, m, b, j, FS, c);
    return;
  }
  typedef typename cplx<T>::type T2;
  constexpr int NSPX = SlotCount<T>::NP;
  const T2* Fp = G.four_p;
  const size_t o = ((size_t)m * G.B + b) * G.g.J + j;
  const T* mc = G.mco;
  const int B = G.B;
  const T xm = (T)m;
  const T tsc = G.jco[(size_t)b * G.g.J + j], dtsc = G.djco[(size_t)b * G.g.J + j];
  const T t1 = tsc * (T)0.25, dt1 = dtsc * (T)0.25;
  const T dte = cfg.forcflag ? dtsc : dtsc * (T)0.5;
  const T t2 = mc[MC_T2 * B + b], ia2 = mc[MC_IA2 * B + b], hPb = mc[MC_HPB * B + b];
  const T dt2 = mc[MC_DT2 * B + b], dia2 = mc[MC_DIA2 * B + b], dhPb = mc[MC_DHPB * B + b];
  const T2 del = Fp[F_DELTA * FS + o], phi = Fp[F_PHI * FS + o], E = Fp[F_E * FS + o];
  const T2 C = Fp[F_C * FS + o], D = Fp[F_D * FS + o];
  const T2 A = Fp[F_A * FS + o], Bm = Fp[F_B * FS + o], Fm = Fp[F_F * FS + o], Gm = Fp[F_G * FS + o];
  const T2 Bf = cadd(Bm, Fm), Af = csub(A, Gm);
  const T2 Beff = cfg.forcflag ? Bf : Bm, Aeff = cfg.forcflag ? Af : A;
  const T dht = dhPb * t1 + hPb * dt1;  // d(hPb t1)
  // Phi
  T2 p1 = cadd(cscale(imul(xm, C), dt1), cscale(del, mc[MC_DDTPB * B + b]));
  p1 = cadd(p1, cscale(imul(xm, Beff), dht));
  c[SP_PHI1] = csub(c[SP_PHI1], p1);
  if (cfg.forcflag) c[SP_PHI1] = cadd(c[SP_PHI1], cscale(Fp[F_PHIF * FS + o], mc[MC_DDT * B + b]));
  c[NSPX + SH_PHI1] = cadd(c[NSPX + SH_PHI1], csub(cscale(D, dt1), cscale(Aeff, dht)));
  c[SP_PHI2] = csub(c[SP_PHI2], cadd(cscale(E, dt2 * hPb + t2 * dhPb), cscale(phi, dia2 * hPb + ia2 * dhPb)));
  // delta
  c[SP_D1] = cadd(c[SP_D1], cscale(imul(xm, Bf), dt1));
  c[NSPX + SH_D1] = cadd(c[NSPX + SH_D1], cscale(Af, dt1));
  const T q = (T)0.5 * (dt1 * ia2 + t1 * dia2);  // d(t1 ia2 / 2)
  T2 d2 = cadd(cscale(cadd(phi, E), dt2), cscale(imul(xm, C), q));
  d2 = csub(d2, cscale(del, mc[MC_DPBA2 * B + b]));
  if (cfg.forcflag) d2 = cadd(d2, cscale(Fp[F_PHIF * FS + o], mc[MC_DPFD * B + b]));
  c[SP_D2] = cadd(c[SP_D2], d2);
  c[NSPX + SH_D2] = cadd(c[NSPX + SH_D2], cscale(D, q));
  // eta
  c[SP_E1] = csub(c[SP_E1], cscale(imul(xm, Aeff), dte));
  c[NSPX + SH_E1] = cadd(c[NSPX + SH_E1], cscale(Beff, dte));
}

// The semi-implicit scheme's coefficient tangents (step_combos_ld scheme 2):
// the shares 1 - gd, 1 - gr (gd = ex / taudrag, gr = ex / taurad under
// relaxation), tstepcoeff, ex Phibar, 2 dt, 1/a^2, the relaxation part of the
// Phi forcing and, on the first step, the drag part of the lagged remainder.
template <typename T>
__device__ __forceinline__ void tangent_coef_terms_si(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                      size_t FS, typename cplx<T>::type* c) {
  typedef typename cplx<T>::type T2;
  constexpr int NSPX = SlotCount<T>::NP;
  const T2* Fp = G.four_p;
  const size_t o = ((size_t)m * G.B + b) * G.g.J + j;
  const T* mc = G.mco;
  const int B = G.B;
  const T xm = (T)m;
  const T tsc = G.jco[(size_t)b * G.g.J + j], dtsc = G.djco[(size_t)b * G.g.J + j];
  const T ex = mc[MC_SIEX * B + b], dex = mc[MC_DSIEX * B + b];
  const T itd = cfg.si_relax ? mc[MC_SIITD * B + b] : (T)0, ditd = cfg.si_relax ? mc[MC_DSIITD * B + b] : (T)0;
  const T itr = cfg.si_relax ? mc[MC_SIITR * B + b] : (T)0, ditr = cfg.si_relax ? mc[MC_DSIITR * B + b] : (T)0;
  const T dgd = dex * itd + ex * ditd, dgr = dex * itr + ex * ditr;
  const T pb = mc[MC_PB * B + b], dpb = (T)2 * mc[MC_DHPB * B + b];
  const T tdt = mc[MC_2DT * B + b], dtdt = (T)2 * mc[MC_DDT * B + b];
  const T ia2 = mc[MC_IA2 * B + b], dia2 = mc[MC_DIA2 * B + b];
  const T2 eta0 = Fp[F_ETA_MID * FS + o], del0 = Fp[F_DELTA_MID * FS + o], phi0 = Fp[F_PHI_MID * FS + o];
  const T2 A = Fp[F_A * FS + o], Bm = Fp[F_B * FS + o], C = Fp[F_C * FS + o], D = Fp[F_D * FS + o];
  const T2 E = Fp[F_E * FS + o];
  T2 Aeff = A, Beff = Bm, PFx = mk<T2>(0, 0), dPFx = mk<T2>(0, 0);
  T2 dAc = mk<T2>(0, 0), dBc = mk<T2>(0, 0);  // coefficient tangents of Aeff, Beff (first step)
  if (cfg.forcflag) {
    T2 Fx, Gx;
    if (cfg.si_relax) {
      const T itd_all = mc[MC_SIITD * B + b], ditd_all = mc[MC_DSIITD * B + b];
      if (cfg.si_lag_init) {
        const T2 U = Fp[F_U * FS + o], V = Fp[F_V * FS + o];
        Fx = cadd(Fp[F_F * FS + o], cscale(U, itd_all));
        Gx = cadd(Fp[F_G * FS + o], cscale(V, itd_all));
        dBc = cscale(U, ditd_all);
        dAc = cscale(V, -ditd_all);
      } else {
        Fx = Fp[F_RU_LAG * FS + o];
        Gx = Fp[F_RV_LAG * FS + o];
      }
      const T2 phi1 = Fp[F_PHI * FS + o];
      PFx = cadd(Fp[F_PHIF * FS + o], cscale(phi1, itr));
      dPFx = cscale(phi1, ditr);
    } else {
      Fx = Fp[F_F * FS + o];
      Gx = Fp[F_G * FS + o];
      PFx = Fp[F_PHIF * FS + o];
    }
    Aeff = csub(A, Gx);
    Beff = cadd(Bm, Fx);
  }
  // eta: (1 - gd) eta0 - tsc i m Aeff ; H: tsc Beff
  c[SP_E1] = csub(c[SP_E1], cadd(cscale(eta0, dgd), cadd(cscale(imul(xm, Aeff), dtsc), cscale(imul(xm, dAc), tsc))));
  c[NSPX + SH_E1] = cadd(c[NSPX + SH_E1], cadd(cscale(Beff, dtsc), cscale(dBc, tsc)));
  // delta: (1 - gd) delta0 + tsc i m Beff ; H: tsc Aeff ; n(n+1): (2 dt E + ex Phi0) / a^2
  c[SP_D1] = cadd(c[SP_D1], csub(cadd(cscale(imul(xm, Beff), dtsc), cscale(imul(xm, dBc), tsc)), cscale(del0, dgd)));
  c[NSPX + SH_D1] = cadd(c[NSPX + SH_D1], cadd(cscale(Aeff, dtsc), cscale(dAc, tsc)));
  const T2 d2a = cadd(cscale(E, dtdt), cscale(phi0, dex)), d2b = cadd(cscale(E, tdt), cscale(phi0, ex));
  c[SP_D2] = cadd(c[SP_D2], cadd(cscale(d2a, ia2), cscale(d2b, dia2)));
  // Phi: (1 - gr) Phi0 - tsc i m C - ex Phibar delta0 + 2 dt PhiFx ; H: tsc D
  T2 p1 = cadd(cscale(phi0, dgr), cscale(imul(xm, C), dtsc));
  p1 = cadd(p1, cscale(del0, dex * pb + ex * dpb));
  c[SP_PHI1] = csub(c[SP_PHI1], p1);
  if (cfg.forcflag) c[SP_PHI1] = cadd(c[SP_PHI1], cadd(cscale(PFx, dtdt), cscale(dPFx, tdt)));
  c[NSPX + SH_PHI1] = cadd(c[NSPX + SH_PHI1], cscale(D, dtsc));
}

// The explicit scheme's coefficient tangents (step_combos_ld scheme 1):
// tstepcoeff, 2 dt Phibar, 2 dt and 1 / taudrag (explicit_tdiff.py:62-78,
// 134-155, 207-226) on the primal state before the step.
template <typename T>
__device__ __forceinline__ void tangent_coef_terms_ex(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                      size_t FS, typename cplx<T>::type* c) {
  typedef typename cplx<T>::type T2;
  constexpr int NSPX = SlotCount<T>::NP;
  const T2* Fp = G.four_p;
  const size_t o = ((size_t)m * G.B + b) * G.g.J + j;
  const T* mc = G.mco;
  const int B = G.B;
  const T xm = (T)m;
  const T t = G.jco[(size_t)b * G.g.J + j], dtc = G.djco[(size_t)b * G.g.J + j];
  const T itd = mc[MC_ITD * B + b], ditd = mc[MC_DITD * B + b];
  const T dt2 = (T)2 * mc[MC_DDT * B + b];                                  // d(2 dt)
  const T d2dtpb = (T)2 * mc[MC_DDTPB * B + b];                             // d(2 dt Phibar)
  const T2 del1 = Fp[F_DELTA * FS + o];
  const T2 A = Fp[F_A * FS + o], Bm = Fp[F_B * FS + o], C = Fp[F_C * FS + o], D = Fp[F_D * FS + o];
  // Phi: phi0 - t i m C - 2 dt Phibar delta1 + 2 dt PhiF ; H: t D
  c[SP_PHI1] = csub(c[SP_PHI1], cadd(cscale(imul(xm, C), dtc), cscale(del1, d2dtpb)));
  if (cfg.forcflag) c[SP_PHI1] = cadd(c[SP_PHI1], cscale(Fp[F_PHIF * FS + o], dt2));
  c[NSPX + SH_PHI1] = cadd(c[NSPX + SH_PHI1], cscale(D, dtc));
  // eta: eta0 - t i m A ; H: t B (plus the forced drag and forcing terms)
  c[SP_E1] = csub(c[SP_E1], cscale(imul(xm, A), dtc));
  c[NSPX + SH_E1] = cadd(c[NSPX + SH_E1], cscale(Bm, dtc));
  if (cfg.forcflag) {
    const T2 U = Fp[F_U * FS + o], V = Fp[F_V * FS + o], Fm = Fp[F_F * FS + o], Gm = Fp[F_G * FS + o];
    const T dti = dtc * itd + t * ditd;  // d(t / taudrag)
    // delta: - t/td i m U + t i m F ; H: t/td V - t G
    c[SP_D1] = cadd(c[SP_D1], csub(cscale(imul(xm, Fm), dtc), cscale(imul(xm, U), dti)));
    c[NSPX + SH_D1] = cadd(c[NSPX + SH_D1], csub(cscale(V, dti), cscale(Gm, dtc)));
    // eta: - t/td i m V + t i m G ; H: t/td U + t F
    c[SP_E1] = cadd(c[SP_E1], csub(cscale(imul(xm, Gm), dtc), cscale(imul(xm, V), dti)));
    c[NSPX + SH_E1] = cadd(c[NSPX + SH_E1], cadd(cscale(U, dti), cscale(Fm, dtc)));
  }
}

// step_combos_ld on the state in global memory
template <typename T>
__device__ __forceinline__ void step_combos(const SpecGroup<T>& G, const StepCfg& cfg, int mode, bool incr, int m,
                                            int b, int j, size_t FS, typename cplx<T>::type* c) {
  const typename cplx<T>::type* F = G.four;
  const size_t o = ((size_t)m * G.B + b) * G.g.J + j;
  step_combos_ld<T>(G, cfg, mode, incr, m, b, j, [&](int f) { return F[f * FS + o]; }, c);
}

// Write-out of one (member, latitude) point of a step at column m: the new curr
// eta, delta, Phi (incremental form: old + increment), the prev carry, the
// Robert-Asselin mid carry (model.py:988-1110) and the winds.  With the RAW
// filter (model.py:1007-1087) the mid level moves by al * d and the new level
// by -an * d; classic RA is al = alpha, an = 0.  The semi-implicit scheme also
// advances its lagged momentum-forcing remainders (model.py:1135-1143).  All
// loads come before the first store: the input and output states may be one
// buffer, so the compiler could not reorder them itself.
// The carries the write-out of a point reads: old curr (3), RA mid (3) and, for
// the semi-implicit scheme, the next lagged remainders Fm + Um / taudrag,
// Gm + Vm / taudrag of the incoming state (2).
template <typename T>
__device__ __forceinline__ void load_step_point(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                                size_t o, typename cplx<T>::type* old, typename cplx<T>::type* mid,
                                                typename cplx<T>::type* lag = nullptr, int b = 0) {
  typedef typename cplx<T>::type T2;
  const T2* Fi = G.four;
  const int cf[3] = {F_ETA, F_DELTA, F_PHI};
  const int rf[3] = {F_ETA_MID, F_DELTA_MID, F_PHI_MID};
  const bool need_old = incr || cfg.write_prev || cfg.ra_mode;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    old[q] = need_old ? Fi[cf[q] * FS + o] : mk<T2>(0, 0);
    mid[q] = cfg.ra_mode == 2 ? Fi[rf[q] * FS + o] : mk<T2>(0, 0);
  }
  if (lag && cfg.scheme == 2) {
    const T itd = G.mco[MC_SIITD * G.B + b];
    lag[0] = cadd(Fi[F_F * FS + o], cscale(Fi[F_U * FS + o], itd));
    lag[1] = cadd(Fi[F_G * FS + o], cscale(Fi[F_V * FS + o], itd));
  }
}

// write_step_point with its carries already loaded (load_step_point)
template <typename T>
__device__ __forceinline__ void store_step_point(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                                 size_t o, T al, T an, const typename cplx<T>::type* nw_in, bool uv,
                                                 typename cplx<T>::type u, typename cplx<T>::type v,
                                                 const typename cplx<T>::type* old,
                                                 const typename cplx<T>::type* mid,
                                                 const typename cplx<T>::type* lag = nullptr, T dal = (T)0,
                                                 T dan = (T)0) {
  typedef typename cplx<T>::type T2;
  T2* Fo = G.four_out;
  const int cf[3] = {F_ETA, F_DELTA, F_PHI};
  const int pf[3] = {F_ETA_PREV, F_DELTA_PREV, F_PHI_PREV};
  const int rf[3] = {F_ETA_MID, F_DELTA_MID, F_PHI_MID};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    T2 nw = nw_in[q];
    if (incr) nw = cadd(old[q], nw);
    if (cfg.write_prev) Fo[pf[q] * FS + o] = old[q];
    if (cfg.ra_mode == 1) Fo[rf[q] * FS + o] = old[q];
    else if (cfg.ra_mode == 2) {
      const T2 d = cadd(csub(mid[q], cscale(old[q], (T)2)), nw);
      Fo[rf[q] * FS + o] = cadd(old[q], cscale(d, al));
      if (cfg.raw) nw = csub(nw, cscale(d, an));
      if (cfg.tl_filter) {
        // primal step of a tangent run: the filter weights' tangents times this
        // displacement (the tangent step, launched before, wrote the rest)
        T2* Ft = G.four_t;
        Ft[rf[q] * FS + o] = cadd(Ft[rf[q] * FS + o], cscale(d, dal));
        if (cfg.raw) Ft[cf[q] * FS + o] = csub(Ft[cf[q] * FS + o], cscale(d, dan));
      }
    }
    Fo[cf[q] * FS + o] = nw;
  }
  if (lag && cfg.scheme == 2) {
    Fo[F_RU_LAG * FS + o] = lag[0];
    Fo[F_RV_LAG * FS + o] = lag[1];
  }
  if (uv) {
    Fo[F_U * FS + o] = u;
    Fo[F_V * FS + o] = v;
  }
}

// load_step_point / store_step_point of the modified-Euler step for the
// R = Rows16 adjacent latitudes j, j+1, ... at offset o of one (m, member),
// with 16-byte accesses (no lagged remainders: scheme 0).  The arithmetic per
// point is that of the single-point forms.
template <typename T, int R = Rows16<typename cplx<T>::type>::N>
__device__ __forceinline__ void load_step_rows(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                               size_t o, typename cplx<T>::type (&old)[3][R],
                                               typename cplx<T>::type (&mid)[3][R]) {
  typedef typename cplx<T>::type T2;
  const T2* Fi = G.four;
  const bool need_old = incr || cfg.write_prev || cfg.ra_mode;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int cf = q == 0 ? F_ETA : q == 1 ? F_DELTA : F_PHI;
    const int rf = q == 0 ? F_ETA_MID : q == 1 ? F_DELTA_MID : F_PHI_MID;
    if (need_old) ld_rows16(Fi + cf * FS + o, old[q]);
    else
#pragma unroll
      for (int e = 0; e < R; ++e) old[q][e] = mk<T2>(0, 0);
    if (cfg.ra_mode == 2) ld_rows16(Fi + rf * FS + o, mid[q]);
    else
#pragma unroll
      for (int e = 0; e < R; ++e) mid[q][e] = mk<T2>(0, 0);
  }
}
template <typename T, int R = Rows16<typename cplx<T>::type>::N>
__device__ __forceinline__ void store_step_rows(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                                size_t o, T al, T an, const typename cplx<T>::type (&nw_in)[3][R],
                                                bool uv, const typename cplx<T>::type (&u)[R],
                                                const typename cplx<T>::type (&v)[R],
                                                const typename cplx<T>::type (&old)[3][R],
                                                const typename cplx<T>::type (&mid)[3][R]) {
  typedef typename cplx<T>::type T2;
  T2* Fo = G.four_out;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int cf = q == 0 ? F_ETA : q == 1 ? F_DELTA : F_PHI;
    const int pf = q == 0 ? F_ETA_PREV : q == 1 ? F_DELTA_PREV : F_PHI_PREV;
    const int rf = q == 0 ? F_ETA_MID : q == 1 ? F_DELTA_MID : F_PHI_MID;
    T2 nw[R], rm[R];
#pragma unroll
    for (int e = 0; e < R; ++e) nw[e] = incr ? cadd(old[q][e], nw_in[q][e]) : nw_in[q][e];
    if (cfg.write_prev) st_rows16(Fo + pf * FS + o, old[q]);
    if (cfg.ra_mode == 1) st_rows16(Fo + rf * FS + o, old[q]);
    else if (cfg.ra_mode == 2) {
#pragma unroll
      for (int e = 0; e < R; ++e) {
        const T2 d = cadd(csub(mid[q][e], cscale(old[q][e], (T)2)), nw[e]);
        rm[e] = cadd(old[q][e], cscale(d, al));
        if (cfg.raw) nw[e] = csub(nw[e], cscale(d, an));
      }
      st_rows16(Fo + rf * FS + o, rm);
    }
    st_rows16(Fo + cf * FS + o, nw);
  }
  if (uv) {
    st_rows16(Fo + F_U * FS + o, u);
    st_rows16(Fo + F_V * FS + o, v);
  }
}

template <typename T>
__device__ __forceinline__ void write_step_point(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                                 size_t o, int b, const typename cplx<T>::type* nw_in, bool uv,
                                                 typename cplx<T>::type u, typename cplx<T>::type v,
                                                 bool tangent = false) {
  typename cplx<T>::type old[3], mid[3], lag[2];
  load_step_point<T>(G, cfg, incr, FS, o, old, mid, lag, b);
  if (tangent && cfg.scheme == 2) {
    // tangent of Fm + Um / taudrag: the primal winds times d(1/taudrag)
    const typename scalar_of<typename cplx<T>::type>::type ditd = G.mco[MC_DSIITD * G.B + b];
    lag[0] = cadd(lag[0], cscale(G.four_p[F_U * FS + o], ditd));
    lag[1] = cadd(lag[1], cscale(G.four_p[F_V * FS + o], ditd));
  }
  const T al = G.mco[(cfg.raw ? MC_RAWM : MC_ALPHA) * G.B + b];
  const T an = cfg.raw ? G.mco[MC_RAWN * G.B + b] : (T)0;
  T dal = (T)0, dan = (T)0;
  if (cfg.tl_filter) {
    dal = G.mco[(cfg.raw ? MC_DRAWM : MC_DALPHA) * G.B + b];
    dan = cfg.raw ? G.mco[MC_DRAWN * G.B + b] : (T)0;
  }
  store_step_point<T>(G, cfg, incr, FS, o, al, an, nw_in, uv, u, v, old, mid, lag, dal, dan);
}

// Residual weights of the initial condition in the physical curr / mid fields
// after a step (the new level is band-limited): classic RA mid = curr + al d,
// RAW also moves the new level by -an d (model.py:988-1087).  With dwc, dwm
// (tangent runs with filter-weight tangents) their tangents along dal (alpha)
// and dwa (williams_alpha) go along, from the same weights before the step.
__device__ __forceinline__ void step_residual_weights_tl(const StepCfg& cfg, double al, double wa, double dal,
                                                         double dwa, double wc, double wm, double& dwc,
                                                         double& dwm) {
  if (cfg.ra_mode == 1) {
    dwm = dwc;
    dwc = 0.0;
  } else if (cfg.ra_mode == 2) {
    const double dw = wm - 2.0 * wc, ddw = dwm - 2.0 * dwc;
    if (cfg.raw) {
      const double m = al * wa, n = al * (1.0 - wa);
      const double dm = dal * wa + al * dwa, dn = dal * (1.0 - wa) - al * dwa;
      dwm = dwc + dm * dw + m * ddw;
      dwc = -(dn * dw + n * ddw);
    } else {
      dwm = dwc + dal * dw + al * ddw;
      dwc = 0.0;
    }
  } else {
    dwc = 0.0;
  }
}
__device__ __forceinline__ void step_residual_weights(const StepCfg& cfg, double al, double wa, double& wc,
                                                      double& wm) {
  if (cfg.ra_mode == 1) {
    wm = wc;
    wc = 0.0;
  } else if (cfg.ra_mode == 2) {
    const double dw = wm - 2.0 * wc;
    if (cfg.raw) {
      wm = wc + (al * wa) * dw;
      wc = -(al * (1.0 - wa)) * dw;
    } else {
      wm = wc + al * dw;
      wc = 0.0;
    }
  } else {
    wc = 0.0;
  }
}

// ----------------------------------------------------------------- adjoint
// Global values the adjoint write-out of one (m, member, latitude) point
// reads, loaded ahead of the stores:
//   modified Euler: the adjoint of the step's curr outputs (incremental form)
//   and the primal delta, Phi, E, A, B, F, G (Phibar gradient);
//   explicit leapfrog: the adjoint of the Fourier prev level after the step
//   (the step moves curr there), and the primal curr delta, U, V (Phibar and
//   taudrag gradients);
//   semi-implicit leapfrog: the adjoint of the filtered mid carry and of the
//   lagged remainders after the step (its parameter gradients are tangent runs).
template <typename T>
struct AdjPointIn {
  // lamY eta, delta, Phi | lambda eta, delta, Phi prev (explicit) | lambda eta, delta, Phi mid (semi-implicit)
  typename cplx<T>::type ly[3];
  // primal delta, Phi, E, A, B, F, G | delta, U, V (explicit) | lambda of the lagged remainders (semi-implicit)
  typename cplx<T>::type px[7];
};

template <typename T>
__device__ __forceinline__ void adj_load_point(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                               size_t o, AdjPointIn<T>& in) {
  typedef typename cplx<T>::type T2;
  const T2 z = mk<T2>(0, 0);
  if (cfg.scheme == 2) {
    const int lf[3] = {F_ETA_MID, F_DELTA_MID, F_PHI_MID};
#pragma unroll
    for (int q = 0; q < 3; ++q) in.ly[q] = G.lam[lf[q] * FS + o];
    in.px[0] = G.lam[F_RU_LAG * FS + o];
    in.px[1] = G.lam[F_RV_LAG * FS + o];
#pragma unroll
    for (int q = 2; q < 7; ++q) in.px[q] = z;
    return;
  }
  if (cfg.scheme == 1) {
    const int lf[3] = {F_ETA_PREV, F_DELTA_PREV, F_PHI_PREV};
    const int pf[3] = {F_DELTA, F_U, F_V};
#pragma unroll
    for (int q = 0; q < 3; ++q) in.ly[q] = G.lam[lf[q] * FS + o];
#pragma unroll
    for (int q = 0; q < 3; ++q) in.px[q] = G.grad ? G.four[pf[q] * FS + o] : z;
#pragma unroll
    for (int q = 3; q < 7; ++q) in.px[q] = z;
    return;
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) in.ly[q] = incr ? G.lamY[q * FS + o] : z;
  const int pf[7] = {F_DELTA, F_PHI, F_E, F_A, F_B, F_F, F_G};
#pragma unroll
  for (int q = 0; q < 7; ++q) in.px[q] = G.grad ? G.four[pf[q] * FS + o] : z;
}

// Transposed combination of the step inputs at one point (adjoint of
// step_combos, modified Euler): from the adjoints of the combined inputs
// ld(q) -- slot order PhiP1, PhiP2, dP1, dP2, eP1, [identity Phi, delta, eta
// when NK = 8], then the H slots PhiH1, dH1, dH2, eH1 -- to the adjoints of the
// state fields: lv = eta, delta, Phi, A, B, C, D, E, PhiF, F, G (adj_field
// order; the other 8 of the 19 fields get zero).  Returns this point's term of
// dL/dPhibar (modEuler_tdiff.py:80-103, 185-193).
__host__ __device__ constexpr int adj_field(int q) {
  return q == 0 ? F_ETA : q == 1 ? F_DELTA : q == 2 ? F_PHI : q == 3 ? F_A : q == 4 ? F_B : q == 5 ? F_C
       : q == 6 ? F_D : q == 7 ? F_E : q == 8 ? F_PHIF : q == 9 ? F_F : F_G;
}
__host__ __device__ constexpr int adj_zero_field(int q) {  // the 8 fields whose adjoint the step zeroes
  return q == 0 ? F_U : q == 1 ? F_V : q == 2 ? F_ETA_PREV : q == 3 ? F_DELTA_PREV : q == 4 ? F_PHI_PREV
       : q == 5 ? F_ETA_MID : q == 6 ? F_DELTA_MID : F_PHI_MID;
}
template <typename T, int NK, typename LD>
__device__ __forceinline__ T adj_point_values(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, int m, int b,
                                              int j, LD ld, const AdjPointIn<T>& in,
                                              typename cplx<T>::type (&lv)[11]) {
  typedef typename cplx<T>::type T2;
  T2 lPhiP1 = ld(0), lPhiP2 = ld(1), ldP1 = ld(2), ldP2 = ld(3), leP1 = ld(4);
  T2 lPhiH1 = ld(NK), ldH1 = ld(NK + 1), ldH2 = ld(NK + 2), leH1 = ld(NK + 3);
  const T* mc = G.mco;
  const int B = G.B;
  const T tsc = G.jco[(size_t)b * G.g.J + j];
  const T dt = mc[MC_DT * B + b];
  T t1 = tsc * (T)0.25, t2 = mc[MC_T2 * B + b];
  T ia2 = mc[MC_IA2 * B + b];
  T hPb = mc[MC_HPB * B + b];
  T te = cfg.forcflag ? tsc : tsc * (T)0.5;
  T xm = (T)m;
  T forc = cfg.forcflag ? (T)1 : (T)0;
  // conj(i*alpha*m) z = -i alpha m z
  auto mimul = [&](T alpha, T2 z) { return imul(-alpha * xm, z); };
  // projection form: curr enters PhiP1, dP1, eP1 with coefficient 1; incremental
  // form: through the identity slots and directly (new = curr + ...)
  T2 idphi = lPhiP1, iddel = ldP1, ideta = leP1;
  if (incr) {
    idphi = cadd(ld(NK > 5 ? 5 : 0), in.ly[2]);
    iddel = cadd(ld(NK > 6 ? 6 : 0), in.ly[1]);
    ideta = cadd(ld(NK > 7 ? 7 : 0), in.ly[0]);
  }
  T2 lphi = csub(cadd(idphi, cscale(ldP2, t2)), cscale(lPhiP2, hPb * ia2));
  T2 ldel = cadd(csub(iddel, cscale(lPhiP1, mc[MC_DTPB * B + b])), cscale(ldP2, -mc[MC_PBA2 * B + b]));
  T2 leta = ideta;
  T2 lC = cadd(mimul(-t1, lPhiP1), mimul(t1 * (T)0.5 * ia2, ldP2));
  T2 lD = cadd(cscale(lPhiH1, t1), cscale(ldH2, t1 * (T)0.5 * ia2));
  T2 lE = cadd(cscale(lPhiP2, -hPb * t2), cscale(ldP2, t2));
  T2 lPF = cscale(cadd(cscale(lPhiP1, dt), cscale(ldP2, mc[MC_PFD * B + b])), forc);
  T2 lBeff = cadd(mimul(-hPb * t1, lPhiP1), cscale(leH1, te));
  T2 lAeff = cadd(cscale(lPhiH1, -hPb * t1), mimul(-te, leP1));
  T2 lBf = mimul(t1, ldP1);
  T2 lAf = cscale(ldH1, t1);
  T2 lA = cadd(lAeff, lAf), lB = cadd(lBeff, lBf);
  T2 lF = cadd(cscale(lBeff, forc), lBf);
  T2 lG = csub(mk<T2>(0, 0), cadd(cscale(lAeff, forc), lAf));
  lv[0] = leta; lv[1] = ldel; lv[2] = lphi; lv[3] = lA; lv[4] = lB; lv[5] = lC; lv[6] = lD;
  lv[7] = lE; lv[8] = lPF; lv[9] = lF; lv[10] = lG;
  if (!G.grad) return (T)0;
  // d(combined inputs)/dPhibar
  const T2 del = in.px[0], phi = in.px[1], E = in.px[2], A = in.px[3], Bm = in.px[4], Fm = in.px[5], Gm = in.px[6];
  T2 Beff = cfg.forcflag ? cadd(Bm, Fm) : Bm, Aeff = cfg.forcflag ? csub(A, Gm) : A;
  T2 dP1 = csub(cscale(del, -dt), cscale(imul(xm, Beff), (T)0.5 * t1));
  T2 dH1 = cscale(Aeff, (T)-0.5 * t1);
  T2 dP2 = cscale(cadd(cscale(E, t2), cscale(phi, ia2)), (T)-0.5);
  T2 dd2 = cscale(del, -ia2);
  return lPhiP1.x * dP1.x + lPhiP1.y * dP1.y + lPhiH1.x * dH1.x + lPhiH1.y * dH1.y + lPhiP2.x * dP2.x +
         lPhiP2.y * dP2.y + ldP2.x * dd2.x + ldP2.y * dd2.y;
}

// Transposed combination of the explicit leapfrog (adjoint of step_combos
// scheme 1; explicit_tdiff.py:62-78, 134-155, 207-226) at one point.  The step
// reads the Fourier prev level (eta0, delta0, Phi0), curr delta, A..D, PhiF,
// F, G, U, V, and moves curr into prev (the unfiltered Fourier carry,
// model.py:1107-1110); so the adjoint of the state before the step is
//   prev: from the P slots directly;  curr: the adjoint of prev after the step
//   (in.ly), plus -2 dt Phibar lambda_PhiP1 on delta;  U, V, A..D, PhiF, F, G:
//   from the slots;  E and the mid carries: zero.
// lv takes the 16 written fields in adj_field_ex order.  Returns this point's
// dL/dPhibar term and adds its dL/dtaudrag term to gtd.
__host__ __device__ constexpr int adj_field_ex(int q) {
  return q == 0 ? F_ETA_PREV : q == 1 ? F_DELTA_PREV : q == 2 ? F_PHI_PREV : q == 3 ? F_ETA : q == 4 ? F_DELTA
       : q == 5 ? F_PHI : q == 6 ? F_U : q == 7 ? F_V : q == 8 ? F_A : q == 9 ? F_B : q == 10 ? F_C
       : q == 11 ? F_D : q == 12 ? F_E : q == 13 ? F_PHIF : q == 14 ? F_F : F_G;
}
template <typename T, int NK, typename LD>
__device__ __forceinline__ T adj_point_values_ex(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                 LD ld, const AdjPointIn<T>& in, typename cplx<T>::type (&lv)[16],
                                                 T& gtd) {
  typedef typename cplx<T>::type T2;
  const T2 lP1 = ld(0), ldP1 = ld(2), leP1 = ld(4);
  const T2 lPH1 = ld(NK), ldH1 = ld(NK + 1), leH1 = ld(NK + 3);
  const T* mc = G.mco;
  const int B = G.B;
  const T t = G.jco[(size_t)b * G.g.J + j];
  const T itd = mc[MC_ITD * B + b];
  const T xm = (T)m;
  const T forc = cfg.forcflag ? (T)1 : (T)0;
  const T2 z = mk<T2>(0, 0);
  // conj(i alpha m) z = -i alpha m z
  auto mimul = [&](T alpha, T2 v) { return imul(-alpha * xm, v); };
  const T2 ldel1 = cscale(lP1, -mc[MC_2DTPB * B + b]);
  lv[0] = leP1;                                    // eta0 (prev)
  lv[1] = ldP1;                                    // delta0
  lv[2] = lP1;                                     // Phi0
  lv[3] = in.ly[0];                                // curr eta -> prev after the step
  lv[4] = cadd(in.ly[1], ldel1);                   // curr delta: carry and -2 dt Phibar delta1
  lv[5] = in.ly[2];                                // curr Phi
  lv[6] = cscale(cadd(mimul(-t * itd, ldP1), cscale(leH1, t * itd)), forc);  // U
  lv[7] = cscale(cadd(cscale(ldH1, t * itd), mimul(-t * itd, leP1)), forc);  // V
  lv[8] = mimul(-t, leP1);                         // A
  lv[9] = cscale(leH1, t);                         // B
  lv[10] = mimul(-t, lP1);                         // C
  lv[11] = cscale(lPH1, t);                        // D
  lv[12] = z;                                      // E
  lv[13] = cscale(lP1, forc * mc[MC_2DT * B + b]); // PhiF
  lv[14] = cscale(cadd(mimul(t, ldP1), cscale(leH1, t)), forc);    // F
  lv[15] = cscale(cadd(cscale(ldH1, -t), mimul(t, leP1)), forc);   // G
  if (!G.grad) return (T)0;
  const T2 del1 = in.px[0], U = in.px[1], V = in.px[2];
  // d(slots)/d(1/taudrag): dP1 -t (i m U), dH1 t V, eP1 -t (i m V), eH1 t U; d(1/taudrag)/dtaudrag = -itd^2
  const T2 dP1 = cscale(imul(xm, U), -t), dH1 = cscale(V, t), eP1 = cscale(imul(xm, V), -t), eH1 = cscale(U, t);
  const T s_itd = ldP1.x * dP1.x + ldP1.y * dP1.y + ldH1.x * dH1.x + ldH1.y * dH1.y + leP1.x * eP1.x +
                  leP1.y * eP1.y + leH1.x * eH1.x + leH1.y * eH1.y;
  gtd += -forc * itd * itd * s_itd;
  // d(PhiP1)/dPhibar = -2 dt delta1
  const T tdt = mc[MC_2DT * B + b];
  return -tdt * (lP1.x * del1.x + lP1.y * del1.y);
}

// Transposed combination of the semi-implicit leapfrog (adjoint of
// step_combos_ld scheme 2, semi_implicit_tdiff.py si_timestep) at one point,
// with the step's carries: the Robert-Asselin update of the filtered mid level
// (mid' = curr + al (mid - 2 curr + new), or curr on the first steps; its new
// level's share enters through lamY) and the lagged remainders (lag' = F + U /
// taudrag of the incoming state).  The step reads the mid level (the n-1 base),
// A..E, PhiF, F, G or the lagged remainders, Phi (relaxation) and, on the first
// step, U, V.  lv takes all 19 fields in field order; the parameter gradients
// of this scheme are tangent runs, so there is no gradient term.
template <typename T, int NK, typename LD>
__device__ __forceinline__ void adj_point_values_si(const SpecGroup<T>& G, const StepCfg& cfg, int m, int b, int j,
                                                    LD ld, const AdjPointIn<T>& in,
                                                    typename cplx<T>::type (&lv)[NFOURIER]) {
  typedef typename cplx<T>::type T2;
  const T2 lP1 = ld(0), lD1 = ld(2), lD2 = ld(3), lE1 = ld(4);
  const T2 lPH1 = ld(NK), lDH1 = ld(NK + 1), lEH1 = ld(NK + 3);
  const T* mc = G.mco;
  const int B = G.B;
  const T tsc = G.jco[(size_t)b * G.g.J + j];
  const T xm = (T)m;
  const bool relax = cfg.si_relax != 0;
  const T forc = cfg.forcflag ? (T)1 : (T)0;
  const T ex = mc[MC_SIEX * B + b];
  const T itd = relax ? mc[MC_SIITD * B + b] : (T)0, itr = relax ? mc[MC_SIITR * B + b] : (T)0;
  const T gd = ex * itd, gr = ex * itr, tdt = mc[MC_2DT * B + b];
  const T ia2 = mc[MC_IA2 * B + b], pb = mc[MC_PB * B + b];
  const T2 z = mk<T2>(0, 0);
  auto mimul = [&](T alpha, T2 v) { return imul(-alpha * xm, v); };  // conj(i alpha m) v
  const T2 lAeff = cadd(mimul(-tsc, lE1), cscale(lDH1, tsc));
  const T2 lBeff = cadd(mimul(tsc, lD1), cscale(lEH1, tsc));
  const T2 lFx = cscale(lBeff, forc), lGx = cscale(lAeff, -forc), lPFx = cscale(lP1, forc * tdt);
  // the Robert-Asselin carry: old curr -> mid' with weight 1 - 2 al (or 1), mid -> mid' with al
  const bool ra2 = cfg.ra_mode == 2;
  const T al = ra2 ? mc[MC_ALPHA * B + b] : (T)0;
  const T c_old = ra2 ? (T)1 - (T)2 * al : (T)1;
  // the lagged remainders after the step, F + U / taudrag of the incoming state (always written)
  const T itd_lag = mc[MC_SIITD * B + b];
  const T2 lRu = in.px[0], lRv = in.px[1];
  const bool from_state = !relax || cfg.si_lag_init;  // Fx, Gx are F, G (+ U, V / taudrag on the first step)
#pragma unroll
  for (int q = 0; q < NFOURIER; ++q) lv[q] = z;
  lv[F_ETA] = cscale(in.ly[0], c_old);
  lv[F_DELTA] = cscale(in.ly[1], c_old);
  lv[F_PHI] = cadd(cscale(in.ly[2], c_old), cscale(lPFx, itr));
  lv[F_U] = cscale(lRu, itd_lag);
  lv[F_V] = cscale(lRv, itd_lag);
  if (relax && cfg.si_lag_init) {
    lv[F_U] = cadd(lv[F_U], cscale(lFx, itd));
    lv[F_V] = cadd(lv[F_V], cscale(lGx, itd));
  }
  lv[F_A] = lAeff;
  lv[F_B] = lBeff;
  lv[F_C] = mimul(-tsc, lP1);
  lv[F_D] = cscale(lPH1, tsc);
  lv[F_E] = cscale(lD2, ia2 * tdt);
  lv[F_PHIF] = lPFx;
  lv[F_F] = from_state ? cadd(lRu, lFx) : lRu;
  lv[F_G] = from_state ? cadd(lRv, lGx) : lRv;
  lv[F_ETA_MID] = cadd(cscale(lE1, (T)1 - gd), cscale(in.ly[0], al));
  lv[F_DELTA_MID] = cadd(csub(cscale(lD1, (T)1 - gd), cscale(lP1, ex * pb)), cscale(in.ly[1], al));
  lv[F_PHI_MID] = cadd(cadd(cscale(lP1, (T)1 - gr), cscale(lD2, ia2 * ex)), cscale(in.ly[2], al));
  // the lagged remainders before the step are read from the carry after the first step
  lv[F_RU_LAG] = from_state ? z : lFx;
  lv[F_RV_LAG] = from_state ? z : lGx;
}

// adj_point_values (modified Euler), adj_point_values_ex (explicit) or
// adj_point_values_si (semi-implicit) written to G.lam at offset o of one
// point.  Returns the point's dL/dPhibar term and adds its dL/dtaudrag term
// (explicit scheme) to gtd.
template <typename T, int NK, typename LD>
__device__ __forceinline__ T adj_store_point(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                             size_t o, int m, int b, int j, LD ld, const AdjPointIn<T>& in,
                                             T& gtd) {
  typedef typename cplx<T>::type T2;
  if (cfg.scheme == 2) {
    T2 lv[NFOURIER];
    adj_point_values_si<T, NK>(G, cfg, m, b, j, ld, in, lv);
    // F_PHI_PREV is neither read nor written by the semi-implicit step: its adjoint passes through
#pragma unroll
    for (int q = 0; q < NFOURIER; ++q)
      if (q != F_PHI_PREV) G.lam[q * FS + o] = lv[q];
    return (T)0;
  }
  if (cfg.scheme == 1) {
    T2 lv[16];
    const T gp = adj_point_values_ex<T, NK>(G, cfg, m, b, j, ld, in, lv, gtd);
#pragma unroll
    for (int q = 0; q < 16; ++q) G.lam[adj_field_ex(q) * FS + o] = lv[q];
    G.lam[F_ETA_MID * FS + o] = mk<T2>(0, 0);
    G.lam[F_DELTA_MID * FS + o] = mk<T2>(0, 0);
    G.lam[F_PHI_MID * FS + o] = mk<T2>(0, 0);
    return gp;
  }
  T2 lv[11];
  const T gp = adj_point_values<T, NK>(G, cfg, incr, m, b, j, ld, in, lv);
#pragma unroll
  for (int q = 0; q < 11; ++q) G.lam[adj_field(q) * FS + o] = lv[q];
  if (!cfg.adj_zeroed)
#pragma unroll
    for (int q = 0; q < 8; ++q) G.lam[adj_zero_field(q) * FS + o] = mk<T2>(0, 0);
  return gp;
}

// adj_load_point / adj_store_point for the R = Rows16 adjacent latitudes
// j0, j0+1, ... at offset o of one (m, member), with 16-byte accesses.
// ld(q, e) is slot q at latitude j0 + e.  Returns the sum of the points'
// dL/dPhibar terms (latitude j0 first).
template <typename T, int R = Rows16<typename cplx<T>::type>::N>
struct AdjRowsIn {
  typename cplx<T>::type ly[3][R];
  typename cplx<T>::type px[7][R];
};
template <typename T, int R = Rows16<typename cplx<T>::type>::N>
__device__ __forceinline__ void adj_load_rows(const SpecGroup<T>& G, bool incr, size_t FS, size_t o,
                                              AdjRowsIn<T, R>& in) {
  typedef typename cplx<T>::type T2;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    if (incr) ld_rows16(G.lamY + q * FS + o, in.ly[q]);
    else
#pragma unroll
      for (int e = 0; e < R; ++e) in.ly[q][e] = mk<T2>(0, 0);
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const int pf = q == 0 ? F_DELTA : q == 1 ? F_PHI : q == 2 ? F_E : q == 3 ? F_A : q == 4 ? F_B : q == 5 ? F_F : F_G;
    if (G.grad) ld_rows16(G.four + pf * FS + o, in.px[q]);
    else
#pragma unroll
      for (int e = 0; e < R; ++e) in.px[q][e] = mk<T2>(0, 0);
  }
}
template <typename T, int NK, typename LD, int R = Rows16<typename cplx<T>::type>::N>
__device__ __forceinline__ T adj_store_rows(const SpecGroup<T>& G, const StepCfg& cfg, bool incr, size_t FS,
                                            size_t o, int m, int b, int j0, LD ld, const AdjRowsIn<T, R>& in) {
  typedef typename cplx<T>::type T2;
  T2 lv[R][11];
  T gp = (T)0;
#pragma unroll
  for (int e = 0; e < R; ++e) {
    AdjPointIn<T> pin;
#pragma unroll
    for (int q = 0; q < 3; ++q) pin.ly[q] = in.ly[q][e];
#pragma unroll
    for (int q = 0; q < 7; ++q) pin.px[q] = in.px[q][e];
    gp += adj_point_values<T, NK>(G, cfg, incr, m, b, j0 + e, [&](int q) { return ld(q, e); }, pin, lv[e]);
  }
#pragma unroll
  for (int q = 0; q < 11; ++q) {
    T2 w[R];
#pragma unroll
    for (int e = 0; e < R; ++e) w[e] = lv[e][q];
    st_rows16(G.lam + adj_field(q) * FS + o, w);
  }
  if (!cfg.adj_zeroed) {
    T2 zz[R];
#pragma unroll
    for (int e = 0; e < R; ++e) zz[e] = mk<T2>(0, 0);
#pragma unroll
    for (int q = 0; q < 8; ++q) st_rows16(G.lam + adj_zero_field(q) * FS + o, zz);
  }
  return gp;
}

}  // namespace swp
